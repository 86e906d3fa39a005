// mcs_device.cuh -- device-side building blocks of the Monte Carlo engine.
//
// Restated algorithms (reference file:line):
//   Ising Metropolis trial        isingLib.c:238-254  (corr = 2(sum_l K s_i s_j - h s_i); accept corr>=0 or exp(corr)>U)
//   O(n) reflection Metropolis    heisenbergLib.c:441-473, xyLib.c:382-409 (ds = -2(s.r)r)
//   onsite delta                  heisenbergLib.c:299-308, xyLib.c:247-254
//   majority block spin           isingLib.c:133-150, heisenbergLib.c:250-262
//   renormalised energy           isingLib.c:152-163 / 388-391, heisenbergLib.c:264-275 / 789-799
//   signed solid angle            heisenbergLib.c:114-127
//   measurement loop              isingLib.c:375-432, heisenbergLib.c:661-831, xyLib.c:589-758
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mcs_internal.h"

namespace mcs {

#define MCS_PI_REF 3.1415926535  // heisenbergLib.c:6

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon et al., SC'11); key = 64-bit seed.
__device__ __forceinline__ uint4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, unsigned long long seed)
{
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return make_uint4(c0, c1, c2, c3);
}
__device__ __forceinline__ uint4 philox_t(uint32_t c0, long long t, uint32_t c3, unsigned long long seed)
{
    return philox(c0, (uint32_t)t, (uint32_t)((unsigned long long)t >> 32), c3, seed);
}
__device__ __forceinline__ float u24(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

// Words of one O(n) Metropolis trial at colour-local index k of colour c in
// sweep t.  An XY trial uses two words (direction, acceptance), so sites k and
// k^1 share one Philox block (counter k >> 1): even k takes words (x, y), odd
// k words (z, w), returned in .x/.y.  A Heisenberg trial uses three words and
// has a block of its own (counter k).
template <int DIM>
__device__ __forceinline__ uint4 on_words(uint32_t k, long long t, uint32_t c, unsigned long long seed)
{
    if (DIM == 2) {
        uint4 w = philox_t(k >> 1, t, c, seed);
        if (k & 1u) { w.x = w.z; w.y = w.w; }
        return w;
    }
    return philox_t(k, t, c, seed);
}

// ------------------------------------------------------------------ geometry
// SQUARE: N = Lx*Ly, Lx, Ly even; hy = Ly/2, half = N/2.  A site of colour c
// with colour-local index k = x*hy + yh sits at (x, y = 2*yh + ((x+c)&1)) and
// has sweep index c*half + k.  Its four neighbours have the other colour.
template <class F>
__device__ __forceinline__ void sq_links(const Rep &R, int c, int x, int yh, F &&f)
{
    const int Lx = R.Lx, Ly = R.Ly, hy = R.hy;
    const int y = 2 * yh + ((x + c) & 1);
    const int base = (1 - c) * R.half;
    const int xp = (x + 1 == Lx) ? 0 : x + 1;
    const int xm = (x == 0) ? Lx - 1 : x - 1;
    const int yp = (y + 1 == Ly) ? 0 : y + 1;
    const int ym = (y == 0) ? Ly - 1 : y - 1;
    f(0, base + xp * hy + yh, R.sq_code[0]);
    f(1, base + xm * hy + yh, R.sq_code[1]);
    f(2, base + x * hy + (yp >> 1), R.sq_code[2]);
    f(3, base + x * hy + (ym >> 1), R.sq_code[3]);
}

// Iterate the links of site v (sweep index): f(slot, neighbour, code).  The
// square lattice slots are +x, -x, +y, -y.
template <int GEOM, class F>
__device__ __forceinline__ void for_links(const Rep &R, int v, F &&f)
{
    if (GEOM == MCS_GEOM_SQUARE) {
        const int c = v >= R.half;
        const int k = v - c * R.half;
        const int x = k / R.hy;
        sq_links(R, c, x, k - x * R.hy, f);
    } else {
        int d = R.deg[v];
        for (int l = 0; l < d; ++l)
            f(l, __ldg(&R.nbr[(size_t)l * R.N + v]), (int)__ldg(&R.lcode[(size_t)l * R.N + v]));
    }
}
template <int GEOM>
__device__ __forceinline__ int link_class(const Rep &R, int v, int l)
{
    if (GEOM == MCS_GEOM_SQUARE) return R.sq_cls[l];
    return R.lcls[(size_t)l * R.N + v];
}

// Walks the colour-local indices k = k0, k0+step, ... of a square lattice
// keeping (x, yh) without divisions.
struct SqWalk {
    int x, yh, dx, dy, hy;
    __device__ __forceinline__ void init(int k0, int step, int hy_)
    {
        hy = hy_;
        x = k0 / hy; yh = k0 - x * hy;
        dx = step / hy; dy = step - dx * hy;
    }
    __device__ __forceinline__ void next()
    {
        yh += dy; x += dx;
        if (yh >= hy) { yh -= hy; ++x; }
    }
};

// ------------------------------------------------------------------ spins
struct Spins {
    signed char *s;     // Ising
    float *x, *y, *z;   // O(n) components (z unused for XY)
};
__device__ __forceinline__ Spins spins_global(const Rep &R)
{
    Spins S;
    S.s = (signed char *)R.spins;
    float *b = (float *)R.spins;
    S.x = b; S.y = b + R.spad; S.z = b + 2 * (size_t)R.spad;
    return S;
}

// ------------------------------------------------------------------ Ising trial
// Threshold-table Metropolis: the neighbour-sign pattern selects an entry whose
// threshold is ceil(exp(corr) * 2^32) (2^32 when corr >= 0); the trial is
// accepted iff the Philox word is below it -- the same decision as
// exp(corr) > w * 2^-32 of the reference rule with U = w * 2^-32.
template <class LINKS>
__device__ __forceinline__ bool ising_trial(const Rep &R, const IsEntry *__restrict__ itab, signed char *s, int v,
                                            int t, uint32_t w, LINKS &&links, int (&dn)[MCS_MAXC], int (&dm)[MCS_MAXT])
{
    int si = s[v];
    int idx = R.ibase[t];
    links([&](int, int j, int code) { if (s[j] > 0) idx += code; });
    const IsEntry e = itab[idx];
    unsigned long long thr = e.thr[si > 0];
    if ((unsigned long long)w < thr) {
        s[v] = (signed char)(-si);
        int nc = e.nc;
        dn[0] += si * (int)(signed char)(nc & 0xff);
        dn[1] += si * (int)(signed char)((nc >> 8) & 0xff);
        dn[2] += si * (int)(signed char)((nc >> 16) & 0xff);
        dn[3] += si * (int)(signed char)((nc >> 24) & 0xff);
#pragma unroll
        for (int q = 0; q < MCS_MAXT; ++q) dm[q] += (q == t) ? si : 0;
        return true;
    }
    return false;
}

// ------------------------------------------------------------------ O(n) trial
// Reflection proposal s' = s - 2(s.r)r with r uniform on the circle / sphere.
// dE = ds . (sum_l J_l s_j) + D.((s+ds)^2 - s^2) - h ds_axis (field along x for
// XY, z for Heisenberg).  Accept dE <= 0 or exp(-beta dE) > U.
// The engine stream defines r = (cos phi, sin phi) (XY) or
// (rho cos phi, rho sin phi, z) (Heisenberg) with phi = 2 pi U.  Every use of r
// -- the reflection s - 2 (s.r) r and the Wolff bond products (s_i.r)(s_j.r)
// -- is unchanged under r -> -r, so the device evaluates -r: the angle
// phi - pi lies in [-pi, pi), where the fast hardware sine and cosine are
// accurate to about 5e-7, and z is negated with it.
template <int DIM>
__device__ __forceinline__ void on_direction(const uint4 &w, float &r0, float &r1, float &r2)
{
    const float two_pi = 6.28318530717958647692f, pi = 3.14159265358979323846f;
    if (DIM == 2) {
        float sp, cp;
        __sincosf(fmaf(two_pi, u24(w.x), -pi), &sp, &cp);
        r0 = cp; r1 = sp; r2 = 0.f;
    } else {
        const float zz = 2.0f * u24(w.x) - 1.0f;
        float sp, cp;
        __sincosf(fmaf(two_pi, u24(w.y), -pi), &sp, &cp);
        const float rho = sqrtf(fmaxf(0.f, 1.f - zz * zz));
        r0 = rho * cp; r1 = rho * sp; r2 = -zz;
    }
}
// The direction itself (random initial spins, where the sign matters).
template <int DIM>
__device__ __forceinline__ void on_direction_exact(const uint4 &w, float &r0, float &r1, float &r2)
{
    if (DIM == 2) {
        float sp, cp;
        sincospif(2.0f * u24(w.x), &sp, &cp);
        r0 = cp; r1 = sp; r2 = 0.f;
    } else {
        const float zz = 2.0f * u24(w.x) - 1.0f;
        float sp, cp;
        sincospif(2.0f * u24(w.y), &sp, &cp);
        const float rho = sqrtf(fmaxf(0.f, 1.f - zz * zz));
        r0 = rho * cp; r1 = rho * sp; r2 = zz;
    }
}

// RR: the replica descriptor, or any type with its fullJ and has_d fields
// (a kernel can pass register copies of them)
template <int DIM, class LINKS, class RR>
__device__ __forceinline__ void on_field(const RR &R, const float *__restrict__ jt, const Spins &S, LINKS &&links,
                                         float &h0, float &h1, float &h2)
{
    h0 = h1 = h2 = 0.f;
    const bool full = R.fullJ;
    links([&](int, int j, int code) {
        const float *M = jt + 9 * code;
        float a = S.x[j], b = S.y[j];
        float c = (DIM == 3) ? S.z[j] : 0.f;
        h0 = fmaf(M[0], a, h0);
        h1 = fmaf(M[1], b, h1);
        if (DIM == 3) h2 = fmaf(M[2], c, h2);
        if (full) {
            h0 = fmaf(M[3], b, h0);
            h1 = fmaf(M[6], a, h1);
            if (DIM == 3) {
                h0 = fmaf(M[4], c, h0);
                h1 = fmaf(M[5], c, h1);
                h2 = fmaf(M[7], a, h2);
                h2 = fmaf(M[8], b, h2);
            }
        }
    });
}

// returns true when accepted; dE (table units, before beta) in *dEout.
// dc: site class (anisotropy vector and |S|).
template <int DIM, class LINKS, class RR>
__device__ __forceinline__ bool on_trial(const RR &R, const float *__restrict__ jt, const float *__restrict__ dt,
                                         const Spins &S, int v, int dc, const uint4 &w, float beta, float h,
                                         LINKS &&links, float *dEout)
{
    float h0, h1, h2;
    on_field<DIM>(R, jt, S, links, h0, h1, h2);
    float r0, r1, r2;
    on_direction<DIM>(w, r0, r1, r2);
    float s0 = S.x[v], s1 = S.y[v];
    float s2 = (DIM == 3) ? S.z[v] : 0.f;
    float sr = s0 * r0 + s1 * r1 + s2 * r2;
    float f = -2.f * sr;
    float d0 = f * r0, d1 = f * r1, d2 = f * r2;
    float dE = d0 * h0 + d1 * h1 + d2 * h2;
    const float *D = dt + 4 * dc;
    if (R.has_d) {
        dE += D[0] * (d0 * (2.f * s0 + d0)) + D[1] * (d1 * (2.f * s1 + d1));
        if (DIM == 3) dE += D[2] * (d2 * (2.f * s2 + d2));
    }
    dE -= h * ((DIM == 3) ? d2 : d0);
    float x = beta * dE;
    uint32_t wa = (DIM == 3) ? w.z : w.y;
    bool acc = (x <= 0.f) || (__expf(-x) > u24(wa));
    if (acc) {
        // the reflection preserves |s| exactly; in FP32 the result is pulled
        // back onto |s| = S so that the length cannot random-walk
        float n0 = s0 + d0, n1 = s1 + d1, n2 = s2 + d2;
        float len2 = n0 * n0 + n1 * n1 + n2 * n2;
        float k = len2 > 0.f ? D[3] * rsqrtf(len2) : 1.f;
        S.x[v] = n0 * k;
        S.y[v] = n1 * k;
        if (DIM == 3) S.z[v] = n2 * k;
        *dEout = dE;
    }
    return acc;
}

// ------------------------------------------------------------------ reductions
// Second stage of the block sums: red[w*K + k] holds warp w's partial of value
// k (nw <= 32 warps).  Warp k sums value k over the warps by an FP64 shuffle
// tree (five dependent adds instead of nw: the device issues FP64 slowly, and
// a block of 1024 threads has 32 partials).  Result in out[0..K-1] for all
// threads after the call.
__device__ __forceinline__ void block_sum_warps(const double *red, double *out, int K, int nw)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwb = (blockDim.x + 31) >> 5;
    for (int k = wid; k < K; k += nwb) {
        double a = lane < nw ? red[lane * K + k] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) out[k] = a;
    }
    __syncthreads();
}
// Sum K doubles over the block in a fixed order.  red: shared [32*K] doubles.
// Result valid in out[0..K-1] (shared) after the call for all threads.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double *red, double *out)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[wid * K + k] = x;
    }
    __syncthreads();
    block_sum_warps(red, out, K, nw);
}
// FP32 inside a warp (32 per-thread partials), FP64 across the warps: the
// device's FP64 rate is a small fraction of its FP32 rate, so per-lane FP64
// arithmetic is kept out of the reduction tree.  Inside the warp the K values
// are reduced by recursive halving (reduce-scatter): at each xor step a lane
// keeps half of its values, adds the partner's copy of that half and sends the
// other half, so K values cost about K shuffles instead of 5 K; afterwards
// lane l holds the warp's sum of value l.
template <int K>
__device__ __forceinline__ void block_sum_f(float (&v)[K], double *red, double *out)
{
    static_assert(K >= 1 && K <= 32, "block_sum_f reduces at most 32 values");
    constexpr int P = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    float x[P];
#pragma unroll
    for (int k = 0; k < P; ++k) x[k] = k < K ? v[k] : 0.f;
    // halving steps over the value set: widths P/2, P/4, ..., 1 at lane bits log2(P)-1 .. 0
#pragma unroll
    for (int w = P / 2; w >= 1; w >>= 1) {
        const bool up = (lane & w) != 0;
#pragma unroll
        for (int j = 0; j < w; ++j) {
            const float send = up ? x[j] : x[j + w];
            const float keep = up ? x[j + w] : x[j];
            x[j] = keep + __shfl_xor_sync(0xffffffffu, send, w);
        }
    }
    // lanes that differ above bit log2(P) hold partial sums of the same value
    float y = x[0];
#pragma unroll
    for (int o = P; o < 32; o <<= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
    const int idx = lane & (P - 1);
    if (lane < P && idx < K) red[wid * K + idx] = (double)y;
    __syncthreads();
    block_sum_warps(red, out, K, nw);
}
template <int K>
__device__ __forceinline__ void block_sum_ll(long long (&v)[K], long long *red, long long *out)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        long long x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[wid * K + k] = x;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        long long a = 0;
        for (int w = 0; w < nw; ++w) a += red[w * K + threadIdx.x];
        out[threadIdx.x] = a;
    }
    __syncthreads();
}

// ------------------------------------------------------------------ measurement helpers
__device__ __forceinline__ void v_norm_ref(float &x, float &y, float &z)
{
    const float l2 = x * x + y * y + z * z;
    if (l2 < 1e-10f) return;  // normalize() leaves vectors shorter than 1e-5 unchanged
    const float r = rsqrtf(l2);
    x *= r; y *= r; z *= r;
}

// getMajoritySpin (O(n)): normalize(sum of cluster spins) * S (signed)
template <int DIM>
__device__ __forceinline__ void on_majority(const Rep &R, const Spins &S, int v, float &mx, float &my, float &mz)
{
    mx = my = mz = 0.f;
    int r = R.rindex[v];
    if (r >= 0) {
        for (int k = 0; k < R.ncl; ++k) {
            int c = __ldg(&R.rcl[(size_t)r * R.ncl + k]);
            mx += S.x[c]; my += S.y[c];
            if (DIM == 3) mz += S.z[c];
        }
    }
    v_norm_ref(mx, my, mz);
    float sv = R.sval[v];
    mx *= sv; my *= sv; mz *= sv;
}

template <int DIM>
__device__ __forceinline__ float on_jdot(const float *M, bool full, float ax, float ay, float az, float bx, float by, float bz)
{
    float e = ax * bx * M[0] + ay * by * M[1];
    if (DIM == 3) e += az * bz * M[2];
    if (full) {
        e += ax * by * M[3] + ay * bx * M[6];
        if (DIM == 3) e += ax * bz * M[4] + ay * bz * M[5] + az * bx * M[7] + az * by * M[8];
    }
    return e;
}

template <int DIM>
__device__ __forceinline__ float on_onsite(const Rep &R, const float *dt, const Spins &S, int v)
{
    float s0 = S.x[v], s1 = S.y[v], s2 = (DIM == 3) ? S.z[v] : 0.f;
    float e = 0.f;
    if (R.has_d) {
        int dc = R.stype ? R.stype[v] : 0;
        const float *D = dt + 4 * dc;
        e = D[0] * s0 * s0 + D[1] * s1 * s1;
        if (DIM == 3) e += D[2] * s2 * s2;
    }
    return e - R.h * ((DIM == 3) ? s2 : s0);
}

// Berg-Luescher solid angle with atan (not atan2), +-pi when |re| < 1e-6.
__device__ __forceinline__ double on_signed_area(const Rep &R, const Spins &S, int a, int b, int c)
{
    if (R.uniform_len) {
        // |S| the same everywhere: s_i.s_j/|S|^2 and s1.(s2 x s3)/|S|^3 share one scale
        const float ax = S.x[a], ay = S.y[a], az = S.z[a];
        const float bx = S.x[b], by = S.y[b], bz = S.z[b];
        const float cx = S.x[c], cy = S.y[c], cz = S.z[c];
        const float l = R.slen[0], il2 = 1.f / (l * l);
        const float s1s2 = (ax * bx + ay * by + az * bz) * il2;
        const float s2s3 = (bx * cx + by * cy + bz * cz) * il2;
        const float s3s1 = (cx * ax + cy * ay + cz * az) * il2;
        const float kx = by * cz - bz * cy, ky = bz * cx - bx * cz, kz = bx * cy - by * cx;
        const float re = 1.f + s1s2 + s2s3 + s3s1;
        const float im = (ax * kx + ay * ky + az * kz) * R.inv_len3;
        if (fabsf(re) < 1e-6f) return im > 0.f ? MCS_PI_REF : -MCS_PI_REF;
        return 2.0 * (double)atanf(__fdividef(im, re));
    }
    float l1 = R.slen[a], l2 = R.slen[b], l3 = R.slen[c];
    float ax = S.x[a], ay = S.y[a], az = S.z[a];
    float bx = S.x[b], by = S.y[b], bz = S.z[b];
    float cx = S.x[c], cy = S.y[c], cz = S.z[c];
    float s1s2 = (ax * bx + ay * by + az * bz) / l1 / l2;
    float s2s3 = (bx * cx + by * cy + bz * cz) / l2 / l3;
    float s3s1 = (cx * ax + cy * ay + cz * az) / l3 / l1;
    float kx = by * cz - bz * cy, ky = bz * cx - bx * cz, kz = bx * cy - by * cx;
    float re = 1.f + s1s2 + s2s3 + s3s1;
    float im = (ax * kx + ay * ky + az * kz) / l1 / l2 / l3;
    if (fabsf(re) < 1e-6f) return im > 0.f ? MCS_PI_REF : -MCS_PI_REF;
    return 2.0 * (double)atanf(im / re);
}

// ------------------------------------------------------------------ O(n) frame over a virtual index range
// Every thread of the block calls this; vb..ve is the index range of this block
// (resident: 0..max list length).  Results in Fout (shared, F_NON doubles),
// valid after return.  red: shared scratch [MCS_RED] doubles.  efull: also sum
// the full energy (bond and onsite parts).  majc: optional shared cache of the
// block spins of the chosen sites ([n_rorb][3]); filled here when given, and
// only usable when the block covers the whole lattice.
// on_frame_inline is the same code inlined into the caller, so that the
// compiler sees which memory the spin arrays live in (the Wolff kernel).
#define MCS_RED (32 * 16 + 32)
template <int DIM, int GEOM>
__device__ __forceinline__ void on_frame_inline(const Rep &R, const float *jt, const float *dt, const Spins &S, int vb,
                                                int ve, bool efull, double *red, double *Fout, float *majc)
{
    const int tid = threadIdx.x, bd = blockDim.x;
    const bool full = R.fullJ;
    // a regular lattice (2x2 blocks on even rows and columns, one spin length,
    // neighbour blocks two sites away) forms its blocks by arithmetic instead
    // of from the lists: block r = (xr, yb) holds sites (x, y), (x, y+1),
    // (x+1, y), (x+1, y+1) with x = 2 xr, y = 2 yb, summed in the lists' order
    const bool reg = R.meas_regular && majc;
    const int hb = R.Ly >> 1, hyr = R.hy;
    if (majc) {
        for (int v = tid; v < R.n_rorb; v += bd) {
            float mx, my, mz;
            if (reg) {
                const int xr = v / hb, yb = v - xr * hb;
                const int a0 = 2 * xr * hyr + yb, a3 = a0 + hyr, a1 = R.half + a0, a2 = R.half + a3;
                mx = S.x[a0] + S.x[a1] + S.x[a2] + S.x[a3];
                my = S.y[a0] + S.y[a1] + S.y[a2] + S.y[a3];
                mz = DIM == 3 ? S.z[a0] + S.z[a1] + S.z[a2] + S.z[a3] : 0.f;
                v_norm_ref(mx, my, mz);
                mx *= R.sval0; my *= R.sval0; mz *= R.sval0;
            } else {
                on_majority<DIM>(R, S, __ldg(&R.rorb[v]), mx, my, mz);
            }
            majc[3 * v] = mx; majc[3 * v + 1] = my; majc[3 * v + 2] = mz;
        }
        __syncthreads();
    }
    auto maj = [&](int site, float &mx, float &my, float &mz) {
        if (majc) {
            int r = R.rindex[site];
            mx = majc[3 * r]; my = majc[3 * r + 1]; mz = majc[3 * r + 2];
        } else {
            on_majority<DIM>(R, S, site, mx, my, mz);
        }
    };
    // pass A: every site (total spin, full energy on re-checks, and the
    // correlated-pair sums when every pair is (v, v)) and circuits
    {
        float a[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        const int e = min(ve, R.N);
        const bool pid = R.pair_identity;
        const bool allp = R.meas_regular != 0;  // a regular lattice: every site is a correlated pair
        for (int v = vb + tid; v < e; v += bd) {
            float sx = S.x[v], sy = S.y[v], sz = DIM == 3 ? S.z[v] : 0.f;
            a[0] += sx; a[1] += sy; a[2] += sz;
            if (pid && (allp || (R.sflag[v] & 1))) { a[6] += sx; a[7] += sy; a[8] += sz; a[9] += sx * sx + sy * sy + sz * sz; }
            if (efull) {
                float h0, h1, h2;
                on_field<DIM>(R, jt, S, [&](auto &&f) { for_links<GEOM>(R, v, f); }, h0, h1, h2);
                a[3] += sx * h0 + sy * h1 + sz * h2;
                a[4] += on_onsite<DIM>(R, dt, S, v);
            }
        }
        if (DIM == 3) {
            const int ec = min(ve, R.ncirc);
            for (int v = vb + tid; v < ec; v += bd)
                a[5] += (float)on_signed_area(R, S, __ldg(&R.circ[3 * v]), __ldg(&R.circ[3 * v + 1]), __ldg(&R.circ[3 * v + 2]));
        }
        block_sum_f<10>(a, red, red + 32 * 16);
        const double *o = red + 32 * 16;
        if (tid < 3) Fout[F_TOT + tid] = o[tid];
        if (tid == 3) Fout[F_EFB] = o[3];
        if (tid == 4) Fout[F_EFO] = o[4];
        if (tid == 5) Fout[F_Q] = o[5];
        if (pid && tid >= 6 && tid < 9) { Fout[F_SI + tid - 6] = o[tid]; Fout[F_SJ + tid - 6] = o[tid]; }
        if (pid && tid == 9) Fout[F_SIJ] = o[9];
        __syncthreads();
    }
    // pass G: orbital groups, four at a time; a group that holds every site
    // is the total spin of pass A
    if (tid < 3 * MCS_MAXG && (R.gall >> (tid / 3)) & 1) Fout[F_G + tid] = Fout[F_TOT + tid % 3];
    for (int g0 = 0; g0 < R.ngroup; g0 += 4) {
        // groups g0..g0+3 that exist and do not hold every site
        const int ng = min(4, R.ngroup - g0);
        const int keep = ~(R.gall >> g0) & ((1 << ng) - 1);
        if (!keep) continue;
        float a[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        const int e = min(ve, R.N);
        for (int v = vb + tid; v < e; v += bd) {
            int m = (R.gmask[v] >> g0) & keep;
            if (!(m & 15)) continue;
            float x = S.x[v], y = S.y[v], z = DIM == 3 ? S.z[v] : 0.f;
#pragma unroll
            for (int g = 0; g < 4; ++g)
                if (m & (1 << g)) { a[3 * g] += x; a[3 * g + 1] += y; a[3 * g + 2] += z; }
        }
        block_sum_f<12>(a, red, red + 32 * 16);
        if (tid < 12 && g0 + tid / 3 < MCS_MAXG && ((keep >> (tid / 3)) & 1)) Fout[F_G + 3 * g0 + tid] = red[32 * 16 + tid];
        __syncthreads();
    }
    // pass B (chosen-site walk): when every correlated pair is (v, v) the pair
    // sums came from pass A; the renormalised sums walk the chosen sites.
    if (R.pair_identity) {
        float a[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = 0.f;
        const int e = min(ve, R.n_rorb);
        for (int r = vb + tid; r < e && reg; r += bd) {
            // regular lattice: every site is a correlated pair, the four
            // neighbour blocks and their coupling classes by direction
            const int xr = r / hb, yb = r - xr * hb, nbx = R.Lx >> 1;
            const float mx = majc[3 * r], my = majc[3 * r + 1], mz = majc[3 * r + 2];
            a[0] += mx; a[1] += my; a[2] += mz; a[3] += mx * mx + my * my + mz * mz;
            const int tg[4] = {(xr + 1 == nbx ? 0 : xr + 1) * hb + yb, (xr == 0 ? nbx - 1 : xr - 1) * hb + yb,
                               xr * hb + (yb + 1 == hb ? 0 : yb + 1), xr * hb + (yb == 0 ? hb - 1 : yb - 1)};
            float corr = 0.f;
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                const int t = tg[d];
                corr += on_jdot<DIM>(jt + 9 * R.rdir_cls[d], full, mx, my, mz, majc[3 * t], majc[3 * t + 1], majc[3 * t + 2]);
            }
            a[4] += corr;
            a[5] += on_onsite<DIM>(R, dt, S, 2 * xr * hyr + yb);
        }
        for (int r = vb + tid; r < e && !reg; r += bd) {
            const int v = __ldg(&R.rorb[r]);
            float mx, my, mz;
            if (majc) { mx = majc[3 * r]; my = majc[3 * r + 1]; mz = majc[3 * r + 2]; }
            else on_majority<DIM>(R, S, v, mx, my, mz);
            if (R.sflag[v] & 1) { a[0] += mx; a[1] += my; a[2] += mz; a[3] += mx * mx + my * my + mz * mz; }
            float corr = 0.f;
            const int d = R.rdeg[r];
            for (int l = 0; l < d; ++l) {
                const int tr = __ldg(&R.rtgt[(size_t)r * R.zmax + l]);  // chosen index of the target
                if (tr < 0) continue;
                float tx, ty, tz;
                if (majc) { tx = majc[3 * tr]; ty = majc[3 * tr + 1]; tz = majc[3 * tr + 2]; }
                else on_majority<DIM>(R, S, __ldg(&R.rorb[tr]), tx, ty, tz);
                corr += on_jdot<DIM>(jt + 9 * R.rjc[(size_t)r * R.zmax + l], full, mx, my, mz, tx, ty, tz);
            }
            a[4] += corr;
            a[5] += on_onsite<DIM>(R, dt, S, v);
        }
        block_sum_f<8>(a, red, red + 32 * 16);
        const double *o = red + 32 * 16;
        if (tid < 3) { Fout[F_SIR + tid] = o[tid]; Fout[F_SJR + tid] = o[tid]; }
        if (tid == 3) Fout[F_SIJR] = o[3];
        if (tid == 4) Fout[F_ERB] = o[4];
        if (tid == 5) Fout[F_ERO] = o[5];
        __syncthreads();
        return;
    }
    // pass B: correlated pairs on both lattices, renormalised energy
    {
        float a[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) a[k] = 0.f;
        const int e = min(ve, R.nlat);
        for (int v = vb + tid; v < e; v += bd) {
            int p = __ldg(&R.cpair[2 * v]), q = __ldg(&R.cpair[2 * v + 1]);
            float px = S.x[p], py = S.y[p], pz = DIM == 3 ? S.z[p] : 0.f;
            float qx = S.x[q], qy = S.y[q], qz = DIM == 3 ? S.z[q] : 0.f;
            a[0] += px; a[1] += py; a[2] += pz; a[3] += qx; a[4] += qy; a[5] += qz;
            a[6] += px * qx + py * qy + pz * qz;
            bool cp = R.rindex[p] >= 0, cq = R.rindex[q] >= 0;
            float mpx = 0, mpy = 0, mpz = 0, mqx = 0, mqy = 0, mqz = 0;
            if (cp) { maj(p, mpx, mpy, mpz); a[7] += mpx; a[8] += mpy; a[9] += mpz; }
            if (cq) {
                if (q == p) { mqx = mpx; mqy = mpy; mqz = mpz; }
                else maj(q, mqx, mqy, mqz);
                a[10] += mqx; a[11] += mqy; a[12] += mqz;
            }
            if (cp && cq) a[13] += mpx * mqx + mpy * mqy + mpz * mqz;
        }
        const int er = min(ve, R.n_rorb);
        for (int v = vb + tid; v < er; v += bd) {
            int j = __ldg(&R.rorb[v]);
            float mx, my, mz;
            if (majc) { mx = majc[3 * v]; my = majc[3 * v + 1]; mz = majc[3 * v + 2]; }
            else on_majority<DIM>(R, S, j, mx, my, mz);
            float corr = 0.f;
            int d = R.rdeg[v];
            for (int l = 0; l < d; ++l) {
                int t = __ldg(&R.rlink[(size_t)v * R.zmax + l]);
                if (t < 0) continue;
                float tx, ty, tz;
                if (R.rindex[t] >= 0) maj(t, tx, ty, tz);
                else { tx = ty = tz = 0.f; }
                corr += on_jdot<DIM>(jt + 9 * R.rjc[(size_t)v * R.zmax + l], full, mx, my, mz, tx, ty, tz);
            }
            a[14] += corr;
            a[15] += on_onsite<DIM>(R, dt, S, j);
        }
        block_sum_f<16>(a, red, red + 32 * 16);
        if (tid < 7) Fout[F_SI + tid] = red[32 * 16 + tid];
        else if (tid < 14) Fout[F_SIR + tid - 7] = red[32 * 16 + tid];
        else if (tid == 14) Fout[F_ERB] = red[32 * 16 + 14];
        else if (tid == 15) Fout[F_ERO] = red[32 * 16 + 15];
        __syncthreads();
    }
}
template <int DIM, int GEOM>
__device__ void on_frame(const Rep &R, const float *jt, const float *dt, const Spins &S, int vb, int ve,
                         bool efull, double *red, double *Fout, float *majc)
{
    on_frame_inline<DIM, GEOM>(R, jt, dt, S, vb, ve, efull, red, Fout, majc);
}

// Fold one measurement frame into the FP64 accumulators.  Follows
// heisenbergLib.c:678-830 / xyLib.c:606-757 in FP64.  The work is split into
// independent items over `nl` lanes (lane < nl; every lane computes the few
// shared scalars itself), so a warp folds a frame in the latency of one item
// rather than of the whole list; nl = 1 is the serial fold.  The lanes must
// see F and R.acc[A_ECUR] (shared memory) before the call.
template <int DIM>
__device__ void on_accumulate_lanes(Rep &R, const double *F, double E, long long m, int lane, int nl)
{
    double *acc = R.acc;
    const double inl = R.inv_nl;
    const double tx = F[F_TOT], ty = F[F_TOT + 1], tz = DIM == 3 ? F[F_TOT + 2] : 0.0;
    const double six = F[F_SI], siy = F[F_SI + 1], siz = DIM == 3 ? F[F_SI + 2] : 0.0;
    const double sjx = F[F_SJ], sjy = F[F_SJ + 1], sjz = DIM == 3 ? F[F_SJ + 2] : 0.0;
    const int G = R.ngroup;
    const int nitem = 12 + (G > 0 ? (G + 1) * (G + 1) : 0);
    for (int it = lane; it < nitem; it += nl) {
        switch (it) {
        case 0: {
            double dx = tx, dy = ty, dz = tz;
            const double len = sqrt(dx * dx + dy * dy + dz * dz);
            if (len >= 1e-5) { const double il = 1.0 / len; dx *= il; dy *= il; dz *= il; }
            acc[A_SIZ] += (dx * six + dy * siy + dz * siz) * inl;
            acc[A_SJZ] += (dx * sjx + dy * sjy + dz * sjz) * inl;
            acc[A_STZ] += (dx * tx + dy * ty + dz * tz) * inl;
            break;
        }
        case 1:
            acc[A_SIH] += (DIM == 3 ? siz : six) * inl;
            acc[A_SJH] += (DIM == 3 ? sjz : sjx) * inl;
            acc[A_STH] += (DIM == 3 ? tz : tx) * inl;
            break;
        case 2: {
            const double M = (DIM == 3) ? sqrt(tx * tx + ty * ty + tz * tz) * inl : sqrt(six * six + siy * siy) * inl;
            const double M2 = M * M;
            acc[A_M2] += M2;
            acc[A_M4] += M2 * M2;
            acc[A_MTOT] += M;
            acc[A_MDM] += acc[A_MPREV] * M;
            acc[A_MPREV] = M;
            if (R.series && m < R.nsweep) {
                double *sr = R.series + (size_t)m * MCS_NSER;
                const double e = E * R.inv_N;
                sr[0] = e; sr[1] = M; sr[2] = (F[F_ERB] * 0.5 + F[F_ERO]) * R.inv_nr; sr[3] = F[F_SIJ] * inl;
            }
            break;
        }
        case 3: acc[A_SI] += fabs(six * inl); acc[A_SI + 1] += fabs(siy * inl); acc[A_SI + 2] += fabs(siz * inl); break;
        case 4: acc[A_SJ] += fabs(sjx * inl); acc[A_SJ + 1] += fabs(sjy * inl); acc[A_SJ + 2] += fabs(sjz * inl); break;
        case 5: acc[A_SIJ] += F[F_SIJ] * inl; break;
        case 6: {
            const double e = E * R.inv_N;
            acc[A_E] += e;
            acc[A_E2] += e * e;
            break;
        }
        case 7:
            for (int k = 0; k < 3; ++k) {
                acc[A_SIR + k] += fabs(F[F_SIR + k] * R.inv_ci);
                acc[A_SJR + k] += fabs(F[F_SJR + k] * R.inv_cj);
            }
            break;
        case 8: acc[A_SIJR] += F[F_SIJR] * R.inv_cij; break;
        case 9: {
            const double er = (F[F_ERB] * 0.5 + F[F_ERO]) * R.inv_nr;
            acc[A_ER] += er;
            acc[A_ER2] += er * er;
            break;
        }
        case 10:
            if (DIM == 3) acc[A_Q] += F[F_Q] * (1.0 / (MCS_PI_REF * 4));
            break;
        case 11: break;
        default: {
            // spin.spin between groups a and b (group G is the whole lattice / N)
            const int idx = it - 12, ga = idx / (G + 1), gb = idx - ga * (G + 1);
            const double ax = ga < G ? F[F_G + 3 * ga] : tx * inl, ay = ga < G ? F[F_G + 3 * ga + 1] : ty * inl;
            const double az = DIM == 3 ? (ga < G ? F[F_G + 3 * ga + 2] : tz * inl) : 0.0;
            const double bx = gb < G ? F[F_G + 3 * gb] : tx * inl, by = gb < G ? F[F_G + 3 * gb + 1] : ty * inl;
            const double bz = DIM == 3 ? (gb < G ? F[F_G + 3 * gb + 2] : tz * inl) : 0.0;
            const double d = ax * bx + ay * by + az * bz;
            acc[A_GRP + idx] += d;
            if (ga == gb) acc[A_GRP + (G + 1) * (G + 1) + ga] += d * d;
        }
        }
    }
}

template <int DIM>
__device__ __forceinline__ void on_accumulate(Rep &R, const double *F, double E, long long m)
{
    on_accumulate_lanes<DIM>(R, F, E, m, 0, 1);
}

// Fold n consecutive measurement frames (indices m0 .. m0+n-1, n <= 32) with
// one warp, keeping the FP64 pipe out of the per-measurement arithmetic (the
// device issues a warp's FP64 instruction over many cycles): the observables of
// each frame are formed in FP32 -- frame j by lane j -- from the frame
// converted once (filled by the caller: frame j at fs + j*MCS_FS_STRIDE,
// entries 0..F_NON), and each FP64 accumulator then takes its n FP64 adds in
// measurement order, all accumulators at once (one per lane).  E[j] = running
// energy after frame j (FP64).  Same formulas as on_accumulate_lanes
// (heisenbergLib.c:678-830, xyLib.c:606-757); the per-measurement values carry
// FP32 rounding (relative 6e-8), the sums over measurements are FP64.
#define MCS_FS_STRIDE (F_NON + 32)
// Neumaier's compensated summation step: s + c carries the running sum, c the
// accumulated rounding errors of the FP32 additions (each recovered exactly).
__device__ __forceinline__ void ksum_add(float &s, float &c, float v)
{
    const float t = s + v;
    c += (fabsf(s) >= fabsf(v)) ? ((s - t) + v) : ((v - t) + s);
    s = t;
}
template <int DIM>
__device__ void on_accumulate_frames(Rep &R, float *fs, const double *E, long long m0, int n, int lane)
{
    double *acc = R.acc;
    if (lane < n) {
        const float *f = fs + lane * MCS_FS_STRIDE;
        float *val = fs + lane * MCS_FS_STRIDE + F_NON;  // [32]: value added to acc[k], k < A_ECUR
        const float inl = R.finv_nl;
        const float tx = f[F_TOT], ty = f[F_TOT + 1], tz = DIM == 3 ? f[F_TOT + 2] : 0.f;
        const float six = f[F_SI], siy = f[F_SI + 1], siz = DIM == 3 ? f[F_SI + 2] : 0.f;
        const float sjx = f[F_SJ], sjy = f[F_SJ + 1], sjz = DIM == 3 ? f[F_SJ + 2] : 0.f;
        float dx = tx, dy = ty, dz = tz;
        const float len = sqrtf(dx * dx + dy * dy + dz * dz);
        if (len >= 1e-5f) { dx /= len; dy /= len; dz /= len; }
        val[A_SIZ] = (dx * six + dy * siy + dz * siz) * inl;
        val[A_SJZ] = (dx * sjx + dy * sjy + dz * sjz) * inl;
        val[A_STZ] = (dx * tx + dy * ty + dz * tz) * inl;
        val[A_SIH] = (DIM == 3 ? siz : six) * inl;
        val[A_SJH] = (DIM == 3 ? sjz : sjx) * inl;
        val[A_STH] = (DIM == 3 ? tz : tx) * inl;
        const float M = (DIM == 3) ? sqrtf(tx * tx + ty * ty + tz * tz) * inl : sqrtf(six * six + siy * siy) * inl;
        const float M2 = M * M;
        val[A_M2] = M2;
        val[A_M4] = M2 * M2;
        val[A_MTOT] = M;
        val[A_MPREV] = 0.f;
        val[A_SI] = fabsf(six * inl); val[A_SI + 1] = fabsf(siy * inl); val[A_SI + 2] = fabsf(siz * inl);
        val[A_SJ] = fabsf(sjx * inl); val[A_SJ + 1] = fabsf(sjy * inl); val[A_SJ + 2] = fabsf(sjz * inl);
        val[A_SIJ] = f[F_SIJ] * inl;
        const float e = (float)(E[lane] * R.inv_N);
        val[A_E] = e;
        val[A_E2] = e * e;
        const float ici = R.finv_ci, icj = R.finv_cj;
        for (int k = 0; k < 3; ++k) {
            val[A_SIR + k] = fabsf(f[F_SIR + k] * ici);
            val[A_SJR + k] = fabsf(f[F_SJR + k] * icj);
        }
        val[A_SIJR] = f[F_SIJR] * R.finv_cij;
        const float er = (f[F_ERB] * 0.5f + f[F_ERO]) * R.finv_nr;
        val[A_ER] = er;
        val[A_ER2] = er * er;
        val[A_Q] = DIM == 3 ? f[F_Q] * (float)(1.0 / (MCS_PI_REF * 4)) : 0.f;
        if (R.series && m0 + lane < R.nsweep) {
            double *sr = R.series + (size_t)(m0 + lane) * MCS_NSER;
            sr[0] = e; sr[1] = M; sr[2] = er; sr[3] = val[A_SIJ];
        }
    }
    __syncwarp();
    if (lane == 0) {  // <M_{m-1} M_m> runs through the frames in order
        float prev = (float)acc[A_MPREV];
        for (int j = 0; j < n; ++j) {
            float *val = fs + j * MCS_FS_STRIDE + F_NON;
            const float M = val[A_MTOT];
            val[A_MDM] = prev * M;
            prev = M;
        }
        acc[A_MPREV] = (double)prev;
    }
    __syncwarp();
    // The n frames' values of one accumulator are summed in FP32 with
    // Neumaier compensation (the sum and its rounding error, together exact
    // to about 2^-48 of the values), then added to the FP64 accumulator with
    // two FP64 adds per fold instead of n: the device issues FP64 at a small
    // fraction of its FP32 rate, and this fold runs while the other CTAs of
    // the cluster wait for it.
    if (lane < A_ECUR && lane != A_MPREV) {
        float sh = 0.f, sl = 0.f;
        for (int j = 0; j < n; ++j) ksum_add(sh, sl, fs[j * MCS_FS_STRIDE + F_NON + lane]);
        acc[lane] = (acc[lane] + (double)sh) + (double)sl;
    }
    const int G = R.ngroup;
    if (G > 0) {
        const float inl = R.finv_nl;
        for (int idx = lane; idx < (G + 1) * (G + 1); idx += 32) {
            const int ga = idx / (G + 1), gb = idx - ga * (G + 1);
            float ah = 0.f, al = 0.f, bh = 0.f, bl = 0.f;
            for (int j = 0; j < n; ++j) {
                const float *f = fs + j * MCS_FS_STRIDE;
                const float ax = ga < G ? f[F_G + 3 * ga] : f[F_TOT] * inl, ay = ga < G ? f[F_G + 3 * ga + 1] : f[F_TOT + 1] * inl;
                const float az = DIM == 3 ? (ga < G ? f[F_G + 3 * ga + 2] : f[F_TOT + 2] * inl) : 0.f;
                const float bx = gb < G ? f[F_G + 3 * gb] : f[F_TOT] * inl, by = gb < G ? f[F_G + 3 * gb + 1] : f[F_TOT + 1] * inl;
                const float bz = DIM == 3 ? (gb < G ? f[F_G + 3 * gb + 2] : f[F_TOT + 2] * inl) : 0.f;
                const float d = ax * bx + ay * by + az * bz;
                ksum_add(ah, al, d);
                ksum_add(bh, bl, d * d);
            }
            acc[A_GRP + idx] = (acc[A_GRP + idx] + (double)ah) + (double)al;
            if (ga == gb) {
                double &a4 = acc[A_GRP + (G + 1) * (G + 1) + ga];
                a4 = (a4 + (double)bh) + (double)bl;
            }
        }
    }
    __syncwarp();
}

// ------------------------------------------------------------------ Ising frame
// Majority sign of the block around v; tie -> Philox word of (a, m, slot).
__device__ __forceinline__ double is_majority(const Rep &R, const signed char *s, int v, const uint4 &w, int slot)
{
    double avg = 0.0;
    int r = R.rindex[v];
    if (r >= 0)
        for (int k = 0; k < R.ncl; ++k) {
            int c = __ldg(&R.rcl[(size_t)r * R.ncl + k]);
            int t = R.stype ? R.stype[c] : 0;
            avg += R.Stype[t] * (double)s[c];
        }
    int tv = R.stype ? R.stype[v] : 0;
    double a = R.Stype[tv];
    if (avg > 0) return a;
    if (avg < 0) return -a;
    uint32_t word = (slot & 3) == 0 ? w.x : (slot & 3) == 1 ? w.y : (slot & 3) == 2 ? w.z : w.w;
    return ((double)word * (1.0 / 4294967296.0) > 0.5) ? a : -a;
}

// Majority sign (single spin length): sign of the sum of the block's signs.
__device__ __forceinline__ int is_majority_sign(const Rep &R, const signed char *s, int v, const uint4 &w, int slot)
{
    int avg = 0;
    int r = R.rindex[v];
    if (r >= 0)
        for (int k = 0; k < R.ncl; ++k) avg += s[__ldg(&R.rcl[(size_t)r * R.ncl + k])];
    if (avg > 0) return 1;
    if (avg < 0) return -1;
    uint32_t word = (slot & 3) == 0 ? w.x : (slot & 3) == 1 ? w.y : (slot & 3) == 2 ? w.z : w.w;
    return ((double)word * (1.0 / 4294967296.0) > 0.5) ? 1 : -1;
}

// Majority sign from a block's sign sum; a tie takes the Philox word of the
// evaluating site and slot (the same decision as is_majority_sign).
// Majority sign of a block with spin sum avg; a tie (avg = 0) is broken by
// word slot & 3 of the Philox block (j, m, 0x3000 + slot >> 2), drawn only
// then: word * 2^-32 > 0.5 exactly when word > 2^31.  The same words and
// decisions as is_majority_from_sum with w drawn up front.
__device__ __forceinline__ int is_majority_lazy(int avg, uint32_t j, long long m, int slot, unsigned long long seed)
{
    if (avg > 0) return 1;
    if (avg < 0) return -1;
    const uint4 w = philox_t(j, m, 0x3000u + (uint32_t)(slot >> 2), seed);
    const uint32_t word = (slot & 3) == 0 ? w.x : (slot & 3) == 1 ? w.y : (slot & 3) == 2 ? w.z : w.w;
    return word > 0x80000000u ? 1 : -1;
}
// Spin sum of the block of site v (0 when v is not a chosen site).
__device__ __forceinline__ int is_block_sum(const Rep &R, const signed char *s, int v)
{
    int avg = 0;
    const int r = R.rindex[v];
    if (r >= 0)
        for (int k = 0; k < R.ncl; ++k) avg += s[__ldg(&R.rcl[(size_t)r * R.ncl + k])];
    return avg;
}
__device__ __forceinline__ int is_majority_from_sum(int avg, const uint4 &w, int slot)
{
    if (avg > 0) return 1;
    if (avg < 0) return -1;
    uint32_t word = (slot & 3) == 0 ? w.x : (slot & 3) == 1 ? w.y : (slot & 3) == 2 ? w.z : w.w;
    return ((double)word * (1.0 / 4294967296.0) > 0.5) ? 1 : -1;
}

// Chosen-site lists of the Ising frame staged in shared memory by a resident
// launch: tgt[r*zmax+l] = chosen index of the l-th renormalised target, -1
// when that target is not a chosen site, -2 when the link does not exist.
struct IsLists {
    const int *rorb;
    const unsigned char *rdeg;
    const int *tgt;
    const unsigned char *kc;
    const int *cp;   // correlated pairs [2*nlat] (nullptr: read R.cpair)
    const int *rcl;  // block members [n_rorb*ncl] (nullptr: read R.rcl)
};

// Ising frame over [vb, ve): pairs, renormalised energy, per-type sign sums,
// full per-class directed bond sums.  Fd (4 doubles) and Fi (MAXT+MAXC ints).
// msum: optional shared cache [n_rorb] of the chosen blocks' sign sums, used
// when the block covers every chosen site (one spin length): each block's sum
// is then formed once per measurement instead of at each of its evaluations.
// il: optional staged lists (with msum).
template <int GEOM>
__device__ void is_frame(const Rep &R, const IsEntry *itab, const signed char *s, int vb, int ve, long long m,
                         double *red, double *Fd, long long *redl, long long *Fi, signed char *msum = nullptr,
                         const IsLists *il = nullptr)
{
    const int tid = threadIdx.x, bd = blockDim.x;
    if (R.is_fast && msum) {
        const int *rcl = (il && il->rcl) ? il->rcl : R.rcl;  // shared-memory copy when staged
        for (int r = tid; r < R.n_rorb; r += bd) {
            int a = 0;
            for (int k = 0; k < R.ncl; ++k) a += s[rcl[(size_t)r * R.ncl + k]];
            msum[r] = (signed char)a;
        }
        __syncthreads();
    }
    if (R.is_fast) {
        // one spin length S0 and <= 4 renormalised coupling values: every sum
        // of the frame is an integer times a constant
        long long c[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) c[k] = 0;
        int e = min(ve, R.nlat);
        const int *cp = (il && il->cp) ? il->cp : R.cpair;  // shared-memory copy when staged
        for (int v = vb + tid; v < e; v += bd) {
            int p = cp[2 * v], q = cp[2 * v + 1];
            int sp = s[p], sq = s[q];
            c[0] += sp; c[1] += sq; c[2] += sp * sq;
        }
        e = min(ve, R.n_rorb);
        // tie-break words are drawn only for tied blocks (is_majority_lazy)
        if (il && msum) {
            const int z = R.zmax;
            for (int v = vb + tid; v < e; v += bd) {
                const int j = il->rorb[v];
                const int mj = is_majority_lazy(msum[v], (uint32_t)j, m, 0, R.seed);
                const int d = il->rdeg[v];
                for (int l = 0; l < d; ++l) {
                    const int tr = il->tgt[v * z + l];
                    if (tr == -2) continue;
                    const int mt = is_majority_lazy(tr >= 0 ? msum[tr] : 0, (uint32_t)j, m, 1 + l, R.seed);
                    const int k = il->kc[v * z + l];
#pragma unroll
                    for (int q = 0; q < 4; ++q) c[3 + q] += (q == k) ? mj * mt : 0;
                }
                c[7] += s[j];
            }
            e = 0;  // done
        }
        for (int v = vb + tid; v < e; v += bd) {
            const int j = __ldg(&R.rorb[v]);
            const int mj = is_majority_lazy(msum ? (int)msum[v] : is_block_sum(R, s, j), (uint32_t)j, m, 0, R.seed);
            const int d = R.rdeg[v];
            for (int l = 0; l < d; ++l) {
                const int slot = 1 + l;
                const int t = __ldg(&R.rlink[(size_t)v * R.zmax + l]);
                if (t < 0) continue;
                int mt;
                if (msum) {
                    const int tr = __ldg(&R.rtgt[(size_t)v * R.zmax + l]);  // chosen index of t, -1: not chosen
                    mt = is_majority_lazy(tr >= 0 ? msum[tr] : 0, (uint32_t)j, m, slot, R.seed);
                } else {
                    mt = is_majority_lazy(is_block_sum(R, s, t), (uint32_t)j, m, slot, R.seed);
                }
                const int k = R.rkc[(size_t)v * R.zmax + l];
#pragma unroll
                for (int q = 0; q < 4; ++q) c[3 + q] += (q == k) ? mj * mt : 0;
            }
            c[7] += s[j];
        }
        e = min(ve, R.N);
        for (int v = vb + tid; v < e; v += bd) {
            int si = s[v];
            int idx = R.ibase[0];
            for_links<GEOM>(R, v, [&](int, int j, int code) { if (s[j] > 0) idx += code; });
            int nc = itab[idx].nc;
            c[8] += si;
            c[12] += si * (int)(signed char)(nc & 0xff);
            c[13] += si * (int)(signed char)((nc >> 8) & 0xff);
            c[14] += si * (int)(signed char)((nc >> 16) & 0xff);
            c[15] += si * (int)(signed char)((nc >> 24) & 0xff);
        }
        block_sum_ll<16>(c, redl, redl + 32 * 16);
        const long long *o = redl + 32 * 16;
        if (tid == 0) {
            const double S0 = R.Stype[0];
            Fd[0] = S0 * (double)o[0];
            Fd[1] = S0 * (double)o[1];
            Fd[2] = S0 * S0 * (double)o[2];
            double er = 0;
            for (int k = 0; k < 4; ++k) er += R.rKv[k] * (double)o[3 + k];
            Fd[3] = S0 * S0 * er / 2 - R.hd * S0 * (double)o[7];
        }
        if (tid < 8) Fi[tid] = o[8 + tid];
        __syncthreads();
        return;
    }
    double a[4] = {0, 0, 0, 0};
    int e = min(ve, R.nlat);
    for (int v = vb + tid; v < e; v += bd) {
        int p = __ldg(&R.cpair[2 * v]), q = __ldg(&R.cpair[2 * v + 1]);
        double sp = R.Stype[R.stype ? R.stype[p] : 0] * (double)s[p];
        double sq = R.Stype[R.stype ? R.stype[q] : 0] * (double)s[q];
        a[0] += sp; a[1] += sq; a[2] += sp * sq;
    }
    e = min(ve, R.n_rorb);
    for (int v = vb + tid; v < e; v += bd) {
        int j = __ldg(&R.rorb[v]);
        uint4 w = philox_t((uint32_t)j, m, 0x3000u, R.seed);
        double mj = is_majority(R, s, j, w, 0);
        double corr = 0;
        int d = R.rdeg[v];
        for (int l = 0; l < d; ++l) {
            int slot = 1 + l;
            if ((slot & 3) == 0) w = philox_t((uint32_t)j, m, 0x3000u + (uint32_t)(slot >> 2), R.seed);
            int t = __ldg(&R.rlink[(size_t)v * R.zmax + l]);
            if (t < 0) continue;
            double mt = is_majority(R, s, t, w, slot);
            corr += R.rK[(size_t)v * R.zmax + l] * mj * mt;
        }
        double sj = R.Stype[R.stype ? R.stype[j] : 0] * (double)s[j];
        a[3] += corr / 2 - R.hd * sj;
    }
    block_sum<4>(a, red, Fd);
    long long c[MCS_MAXT + MCS_MAXC];
#pragma unroll
    for (int k = 0; k < MCS_MAXT + MCS_MAXC; ++k) c[k] = 0;
    e = min(ve, R.N);
    for (int v = vb + tid; v < e; v += bd) {
        int si = s[v];
        int t = R.stype ? R.stype[v] : 0;
        int idx = R.ibase[t];
        for_links<GEOM>(R, v, [&](int, int j, int code) { if (s[j] > 0) idx += code; });
        int nc = itab[idx].nc;
#pragma unroll
        for (int q = 0; q < MCS_MAXT; ++q) c[q] += (q == t) ? si : 0;
        c[MCS_MAXT + 0] += si * (int)(signed char)(nc & 0xff);
        c[MCS_MAXT + 1] += si * (int)(signed char)((nc >> 8) & 0xff);
        c[MCS_MAXT + 2] += si * (int)(signed char)((nc >> 16) & 0xff);
        c[MCS_MAXT + 3] += si * (int)(signed char)((nc >> 24) & 0xff);
    }
    block_sum_ll<MCS_MAXT + MCS_MAXC>(c, redl, Fi);
}

// Fold one Ising measurement (one thread).  isingLib.c:388-431.
__device__ inline void is_accumulate(Rep &R, const double *Fd, const long long *Fi, int last_sign, long long m)
{
    double *acc = R.acc;
    long long *ic = R.icnt;
    double Mtrue = 0;
    for (int t = 0; t < R.ntype; ++t) Mtrue += R.Stype[t] * (double)Fi[t];
    // exact check: incremental bookkeeping vs full recompute
    bool ok = true;
    for (int c = 0; c < MCS_MAXC; ++c) ok &= (Fi[MCS_MAXT + c] - ic[C_N0 + c]) == ic[C_DN + c];
    for (int t = 0; t < MCS_MAXT; ++t) ok &= (Fi[t] - ic[C_M0 + t]) == ic[C_DM + t];
    if (!ok && R.exact_ok) ic[C_MISM] += 1;
    double e_rep;
    if (R.alg == 0) {
        double Einc = 0;
        for (int c = 0; c < R.nclass; ++c) Einc += 0.5 * R.Q[c] * (double)ic[C_DN + c];
        for (int t = 0; t < R.ntype; ++t) Einc -= R.hd * R.Stype[t] * (double)ic[C_DM + t];
        if (R.offset_energy) e_rep = Einc - acc[B_EMEAS0];
        else {
            double E0 = 0;
            for (int c = 0; c < R.nclass; ++c) E0 += 0.5 * R.Q[c] * (double)ic[C_N0 + c];
            for (int t = 0; t < R.ntype; ++t) E0 -= R.hd * R.Stype[t] * (double)ic[C_M0 + t];
            e_rep = E0 + Einc;
        }
    } else {
        double Eabs = 0;
        for (int c = 0; c < R.nclass; ++c) Eabs += 0.5 * R.Q[c] * (double)Fi[MCS_MAXT + c];
        for (int t = 0; t < R.ntype; ++t) Eabs -= R.hd * R.Stype[t] * (double)Fi[t];
        e_rep = (ic[C_ACC_MEAS] || !R.offset_energy) ? Eabs : 0.0;
    }
    double ts = Mtrue - R.ts_const;
    if (R.ts_wolff_last) ts -= R.Stype[R.stype ? R.stype[R.last_site] : 0] * (double)last_sign;
    acc[B_STOT] += ts;
    double M = Fd[0] * R.inv_nl;
    acc[B_M2] += M * M;
    acc[B_M4] += M * M * M * M;
    acc[B_MTOT] += M;
    acc[B_MDM] += acc[B_MPREV] * M;
    acc[B_MPREV] = M;
    acc[B_SI] += fabs(Fd[0]) * R.inv_nl;
    acc[B_SJ] += fabs(Fd[1]) * R.inv_nl;
    acc[B_SIJ] += Fd[2] * R.inv_nl;
    double e = e_rep * R.inv_N, er = Fd[3] * R.inv_nr;
    acc[B_E] += e;
    acc[B_ER] += er;
    acc[B_E2] += e * e;
    acc[B_ER2] += er * er;
    if (R.series && m < R.nsweep) {
        double *s = R.series + (size_t)m * MCS_NSER;
        s[0] = e; s[1] = M; s[2] = er; s[3] = Fd[2] * R.inv_nl;
    }
}

// Spin frame `fw`, site v (sweep index) from local index li of S: Ising signs
// as int8 ([N] per frame), O(n) components as FP32 ([N][dim] per frame), stored
// straight into the replica's page-locked host buffer (mapped into the device),
// so a snapshot leaves the device as it is taken and holds no device memory.
template <int DIM>
__device__ __forceinline__ void frame_store(const Rep &R, int fw, int v, const Spins &S, int li)
{
    if (DIM == 1) {
        ((signed char *)R.frame_buf)[(size_t)fw * R.N + v] = S.s[li];
    } else {
        float *fb = (float *)R.frame_buf + ((size_t)fw * R.N + v) * DIM;
        fb[0] = S.x[li];
        fb[1] = S.y[li];
        if (DIM == 3) fb[2] = S.z[li];
    }
}

__device__ __forceinline__ bool measures_after(const Rep &R, long long u)
{
    return u >= R.units_thermal && ((u - R.units_thermal + 1) % R.upm) == 0;
}

}  // namespace mcs
