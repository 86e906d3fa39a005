// mcs_engine.cpp -- host engine and C ABI of libmcsgpu.so.
//
// A Batch holds replicas (independent solves).  Each replica owns one device
// arena (descriptor arrays, tables, spins, FP64 accumulators).  At run time
// the replicas are grouped by (model dimension, geometry, algorithm, schedule):
//   resident groups: one persistent launch per chunk of units (one CTA per
//                    replica, lattice in shared memory);
//   tiled groups   : lockstep units, one launch per colour + measure + finalize,
//                    captured in a CUDA graph and replayed;
//   plain          : the tiled sequence for one replica at a time without
//                    graphs (the one-solve-per-launch-sequence baseline).
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mcsgpu.h"
#include "mcs_engine.h"
#include "mcs_internal.h"
#include "mcs_model.h"

namespace mcs {

static thread_local std::string g_err;

// The batch and the server run every launch group on its own stream, side by
// side; with the runtime's default of 8 hardware connections, groups beyond
// the eighth share a connection and wait for one another.  Raised to 32 when
// the library loads, unless the process has set it (it must be set before the
// device context is created).
__attribute__((constructor)) static void mcs_raise_connections()
{
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}
void set_error(const std::string &s) { g_err = s; }
const std::string &get_error() { return g_err; }

#define CUDA_TRY(x)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #x);         \
            return MCS_ECUDA;                                                                    \
        }                                                                                        \
    } while (0)

// ------------------------------------------------------------------ arena builder
struct ArenaBuilder {
    // offsets are handed out as pieces are added; the bytes are gathered into
    // one allocation by finish() (the pieces' storage must live until then)
    struct Piece {
        size_t off;
        const void *data;
        size_t bytes;
    };
    std::vector<Piece> pieces;
    size_t size = 256;  // offset 0 is never used
    size_t add(const void *data, size_t bytes)
    {
        size_t off = (size + 255) & ~(size_t)255;
        pieces.push_back({off, data, bytes});
        size = off + bytes;
        return off;
    }
    template <class T> size_t addv(const std::vector<T> &v) { return add(v.empty() ? nullptr : v.data(), v.size() * sizeof(T)); }
    std::vector<unsigned char> finish() const
    {
        std::vector<unsigned char> host(size, 0);  // pieces without data and the gaps stay zero
        for (const Piece &q : pieces)
            if (q.data && q.bytes) memcpy(host.data() + q.off, q.data, q.bytes);
        return host;
    }
};

// Arenas come from the device's default memory pool, kept cached by the
// process (release threshold raised once per device): batches and served
// requests allocate and free an arena each, and a pooled allocation costs a
// fraction of a cudaMalloc.
static std::mutex g_pool_mutex;
static bool g_pool_ready[64];

static void pool_ready(int device)
{
    if (device < 0 || device >= 64) return;
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pool_ready[device]) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t thr = ~0ULL;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
        cudaGetLastError();
        g_pool_ready[device] = true;
    }
}

static int arena_alloc(int device, size_t bytes, void **out, cudaStream_t st)
{
    pool_ready(device);
    CUDA_TRY(cudaMallocAsync(out, bytes, st));
    return MCS_OK;
}

// The batch's own device buffers (descriptors, a lattice's index lists, group
// tables) come from the same pool on the legacy stream: cudaMalloc and
// cudaFree synchronise the device, and creating and destroying a batch would
// pay that for each buffer.  Every user of such a buffer is ordered after its
// allocation (the legacy stream is synchronised before the buffer is handed
// out), and every free comes after the batch's streams were synchronised.
static cudaError_t buf_alloc(int device, void **out, size_t bytes)
{
    pool_ready(device);
    cudaError_t e = cudaMallocAsync(out, std::max<size_t>(bytes, 16), 0);
    // the buffer is ready for any stream once the legacy stream is (our
    // streams are non-blocking: this waits for nothing of theirs)
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    return e;
}
static void buf_free(void *p)
{
    if (p) cudaFreeAsync(p, 0);
}

Replica::~Replica()
{
    if (arena) {
        cudaSetDevice(device);
        cudaFreeAsync(arena, 0);
    }
    if (frames_host) cudaFreeHost(frames_host);
}

size_t replica_acc_count(const HostModel &m)
{
    if (m.dim == 1) return B_NACC;
    int G = m.ngroup;
    return A_GRP + (size_t)(G + 1) * (G + 1) + (G + 1);
}

SharedLists::~SharedLists()
{
    buf_free(d);
}

// One allocation holding the index arrays of a lattice (the pieces a replica
// compiled from its template takes unchanged), uploaded once.
int make_shared_lists(const HostModel &m, int device, std::unique_ptr<SharedLists> *out)
{
    ArenaBuilder A;
    std::unique_ptr<SharedLists> sh(new SharedLists());
    size_t o_nbr = 0, o_lcode = 0, o_deg = 0;
    if (m.geom == MCS_GEOM_ELL) { o_nbr = A.addv(m.nbr); o_lcode = A.addv(m.lcode); o_deg = A.addv(m.deg); }
    const size_t o_stype = A.addv(m.stype), o_cp = A.addv(m.cpair), o_rorb = A.addv(m.rorb), o_rcl = A.addv(m.rcl),
                 o_rlink = A.addv(m.rlink), o_rjc = A.addv(m.rjc), o_rdeg = A.addv(m.rdeg), o_rindex = A.addv(m.rindex),
                 o_circ = A.addv(m.circ), o_slen = A.addv(m.slen), o_sval = A.addv(m.sval), o_gmask = A.addv(m.gmask),
                 o_sflag = A.addv(m.sflag), o_rtgt = A.addv(m.rtgt);
    std::vector<unsigned char> img = A.finish();
    CUDA_TRY(cudaSetDevice(device));
    CUDA_TRY(buf_alloc(device, &sh->d, img.size()));
    sh->bytes = img.size();
    CUDA_TRY(cudaMemcpy(sh->d, img.data(), img.size(), cudaMemcpyHostToDevice));
    unsigned char *b = (unsigned char *)sh->d;
    if (m.geom == MCS_GEOM_ELL) {
        sh->nbr = (const int *)(b + o_nbr);
        sh->lcode = (const unsigned short *)(b + o_lcode);
        sh->deg = b + o_deg;
    }
    sh->stype = b + o_stype;
    sh->cpair = (const int *)(b + o_cp); sh->rorb = (const int *)(b + o_rorb); sh->rcl = (const int *)(b + o_rcl);
    sh->rlink = (const int *)(b + o_rlink); sh->rjc = (const unsigned short *)(b + o_rjc); sh->rdeg = b + o_rdeg;
    sh->rindex = (const int *)(b + o_rindex); sh->circ = (const int *)(b + o_circ);
    sh->slen = (const float *)(b + o_slen); sh->sval = (const float *)(b + o_sval);
    sh->gmask = b + o_gmask; sh->sflag = b + o_sflag; sh->rtgt = (const int *)(b + o_rtgt);
    *out = std::move(sh);
    return MCS_OK;
}

int build_replica(const mcs_problem *p, const mcs_options *o, Replica *r, bool upload, const ModelTemplate *tmpl,
                  bool *reused, const SharedLists *shared)
{
    std::string err;
    bool re = false;
    int rc = compile_model(p, o, &r->hm, &err, tmpl, &re);
    if (reused) *reused = re;
    if (rc != MCS_OK) { set_error(err); return rc; }
    const HostModel &m = r->hm;
    // a replica compiled from its lattice's template reads the batch's shared
    // copy of the index arrays; its arena holds only its own values and state
    const bool share = shared && re && m.dim > 1;
    r->shared = share ? shared : nullptr;
    static const std::vector<int> no_i;
    static const std::vector<uint16_t> no_u16;
    static const std::vector<uint8_t> no_u8;
    static const std::vector<float> no_f;
    r->record_series = o && o->record_series;
    r->requested_schedule = o ? o->schedule : 0;
    r->recheck = (o && o->recheck_every > 0) ? o->recheck_every : 32;
    ArenaBuilder A;
    size_t o_nbr = 0, o_lcode = 0, o_lcls = 0, o_deg = 0, o_stype = 0, o_jt = 0, o_jt64 = 0, o_dt = 0, o_it = 0;
    if (m.geom == MCS_GEOM_ELL) {
        o_nbr = A.addv(share ? no_i : m.nbr);
        o_lcode = A.addv(share ? no_u16 : m.lcode);
        o_deg = A.addv(share ? no_u8 : m.deg);
    }
    if (m.dim == 1) o_lcls = A.addv(m.lcls);
    o_stype = A.addv(share ? no_u8 : m.stype);
    if (m.dim > 1) { o_jt = A.addv(m.jtab); o_jt64 = A.addv(m.jtab64); o_dt = A.addv(m.dtab); }
    else o_it = A.addv(m.itab);
    size_t o_cp = A.addv(share ? no_i : m.cpair), o_rorb = A.addv(share ? no_i : m.rorb),
           o_rcl = A.addv(share ? no_i : m.rcl), o_rlink = A.addv(share ? no_i : m.rlink);
    size_t o_rjc = 0, o_rK = 0;
    if (m.dim > 1) o_rjc = A.addv(share ? no_u16 : m.rjc);
    else o_rK = A.addv(m.rK);
    size_t o_rkc = m.dim == 1 ? A.addv(m.rkc) : 0;
    size_t o_rdeg = A.addv(share ? no_u8 : m.rdeg), o_rindex = A.addv(share ? no_i : m.rindex),
           o_circ = A.addv(share ? no_i : m.circ);
    size_t o_slen = A.addv(share ? no_f : m.slen), o_sval = A.addv(share ? no_f : m.sval),
           o_gmask = A.addv(share ? no_u8 : m.gmask);
    size_t o_sflag = A.addv(share ? no_u8 : m.sflag), o_rtgt = A.addv(share ? no_i : m.rtgt);
    int spad = (m.N + 31) & ~31;
    size_t o_spins;
    std::vector<float> sp;  // O(n) spins padded per component (lives until A.finish())
    if (m.dim == 1) o_spins = A.addv(m.init_sigma);
    else {
        sp.assign((size_t)m.dim * spad, 0.f);
        for (int c = 0; c < m.dim; ++c)
            memcpy(sp.data() + (size_t)c * spad, m.init_vec.data() + (size_t)c * m.N, sizeof(float) * m.N);
        o_spins = A.addv(sp);
    }
    size_t nacc = replica_acc_count(m);
    size_t o_acc = A.add(nullptr, nacc * sizeof(double));
    size_t o_icnt = A.add(nullptr, C_NINT * sizeof(long long));
    size_t o_stats = A.add(nullptr, S_NSTAT * sizeof(long long));
    size_t o_series = 0;
    if (r->record_series) o_series = A.add(nullptr, (size_t)m.nsweep * MCS_NSER * sizeof(double));
    // spin frames live in page-locked host memory (upload_replica), not in the arena
    r->frames_bytes = m.frames > 0 ? (size_t)m.frames * m.N * (m.dim == 1 ? 1 : m.dim * sizeof(float)) : 0;
    size_t o_wbits = 0, o_wq = 0, o_wmaj = 0;
    if (m.alg == 1) {
        o_wbits = A.add(nullptr, ((size_t)(m.N + 31) / 32) * sizeof(unsigned));
        o_wq = A.add(nullptr, (size_t)m.N * sizeof(int));
        if (m.dim > 1) o_wmaj = A.add(nullptr, (size_t)m.n_rorb * 3 * sizeof(float));
    }
    r->bytes = A.size;
    // the descriptor holds arena offsets until upload_replica() relocates them
    auto P = [](size_t off) { return (void *)(uintptr_t)off; };
    Rep &R = r->rep;
    memset(&R, 0, sizeof R);
    R.model = m.model; R.dim = m.dim; R.geom = m.geom; R.alg = m.alg;
    R.N = m.N; R.zmax = m.zmax; R.ncol = m.ncol; R.Ly = m.Ly;
    R.Lx = m.Lx; R.hy = m.Ly / 2; R.half = m.N / 2;
    for (int d = 0; d < 4; ++d) { R.sq_code[d] = m.sq_code[d]; R.sq_cls[d] = m.sq_cls[d]; }
    for (int c = 0; c <= m.ncol; ++c) R.col_start[c] = m.col_start[c];
    if (m.geom == MCS_GEOM_ELL) {
        R.nbr = (const int *)P(o_nbr);
        R.lcode = (const unsigned short *)P(o_lcode);
        R.deg = (const unsigned char *)P(o_deg);
    }
    if (m.dim == 1) R.lcls = (const unsigned char *)P(o_lcls);
    R.stype = (const unsigned char *)P(o_stype);
    if (m.dim > 1) {
        R.jtab = (const float *)P(o_jt); R.jtab64 = (const double *)P(o_jt64);
        R.njc = m.njc; R.fullJ = m.fullJ;
        R.dtab = (const float *)P(o_dt); R.ndc = m.ndc; R.has_d = m.has_d;
    } else {
        R.itab = (const IsEntry *)P(o_it); R.nite = (int)m.itab.size(); R.ntype = m.ntype;
        for (int t = 0; t < MCS_MAXT; ++t) { R.ibase[t] = m.ibase[t]; R.Stype[t] = m.Stype[t]; }
        for (int c = 0; c < MCS_MAXC; ++c) {
            R.Q[c] = m.Q[c];
            R.wthr[c][0] = m.wthr[c][0]; R.wthr[c][1] = m.wthr[c][1];
        }
        R.nclass = m.nclass; R.exact_ok = m.exact_ok;
    }
    R.beta = 1.0f; R.h = (float)m.h; R.hd = m.h;
    R.fp64 = 0;
    R.seed = m.seed;
    R.nlat = m.nlat; R.cpair = (const int *)P(o_cp);
    R.n_rorb = m.n_rorb; R.ncl = m.ncl;
    R.rorb = (const int *)P(o_rorb); R.rcl = (const int *)P(o_rcl); R.rlink = (const int *)P(o_rlink);
    if (m.dim > 1) R.rjc = (const unsigned short *)P(o_rjc);
    else {
        R.rK = (const double *)P(o_rK);
        R.rkc = (const unsigned char *)P(o_rkc);
        R.is_fast = m.is_fast;
        for (int k = 0; k < 4; ++k) R.rKv[k] = m.rKv[k];
    }
    R.rdeg = (const unsigned char *)P(o_rdeg);
    R.rindex = (const int *)P(o_rindex);
    R.ncirc = m.ncirc; R.circ = (const int *)P(o_circ);
    R.slen = (const float *)P(o_slen); R.sval = (const float *)P(o_sval);
    R.ngroup = m.ngroup; R.gmask = (const unsigned char *)P(o_gmask);
    R.ci = m.ci; R.cj = m.cj; R.cij = m.cij;
    R.inv_nl = 1.0 / m.nlat; R.inv_N = 1.0 / m.N;
    R.inv_ci = 1.0 / m.ci; R.inv_cj = 1.0 / m.cj; R.inv_cij = 1.0 / m.cij; R.inv_nr = 1.0 / m.n_rorb;
    R.finv_nl = (float)R.inv_nl; R.finv_N = (float)R.inv_N; R.finv_ci = (float)R.inv_ci;
    R.finv_cj = (float)R.inv_cj; R.finv_cij = (float)R.inv_cij; R.finv_nr = (float)R.inv_nr;
    R.nacc = (int)replica_acc_count(m);
    {
        bool uni = true;
        for (int k = 0; k < m.N && uni; ++k) uni = m.slen[k] == m.slen[0];
        R.uniform_len = uni && m.slen[0] > 0;
        R.inv_len3 = R.uniform_len ? 1.0f / (m.slen[0] * m.slen[0] * m.slen[0]) : 0.f;
    }
    R.pair_identity = m.pair_identity;
    R.gall = m.gall;
    R.meas_regular = m.meas_regular;
    R.sval0 = m.sval.empty() ? 0.f : m.sval[0];
    for (int d = 0; d < 4; ++d) R.rdir_cls[d] = m.rdir_cls[d];
    for (int k = 0; k < 16; ++k) R.rdir_slot[k] = (unsigned char)m.rdir_slot[k];
    R.sflag = (const unsigned char *)P(o_sflag);
    R.rtgt = (const int *)P(o_rtgt);
    R.units_thermal = m.units_thermal; R.units_total = m.units_total; R.nsweep = m.nsweep; R.upm = m.upm;
    R.frames = m.frames; R.frame_every = m.frame_every;
    R.recheck = r->recheck;
    R.ts_const = m.ts_const; R.ts_wolff_last = m.ts_wolff_last; R.last_site = m.last_site;
    R.offset_energy = m.offset_energy;
    R.rinit = m.device_random_init;
    R.spins = P(o_spins); R.spad = spad;
    R.acc = (double *)P(o_acc);
    R.series = r->record_series ? (double *)P(o_series) : nullptr;
    R.frame_buf = nullptr;  // set by upload_replica
    R.icnt = (long long *)P(o_icnt);
    R.stats = (long long *)P(o_stats);
    if (m.alg == 1) {
        R.wbits = (unsigned *)P(o_wbits); R.wqueue = (int *)P(o_wq);
        if (m.dim > 1) R.wmaj = (float *)P(o_wmaj);
    }
    R.u0 = 0; R.u = 0; R.m = 0;
    R.u_stop = m.units_total; R.quota = 0;
    r->acc_off = o_acc; r->icnt_off = o_icnt; r->stats_off = o_stats; r->series_off = o_series;
    r->spins_off = o_spins;
    r->nacc = nacc;
    r->staging = A.finish();
    if (upload) return upload_replica(r);
    return MCS_OK;
}

// Device allocation, upload (through page-locked memory) and relocation of
// the descriptor's arena offsets to device pointers.
int upload_replica(Replica *r)
{
    if (r->arena) return MCS_OK;
    CUDA_TRY(cudaSetDevice(r->device));
    {
        static thread_local void *pinned = nullptr;
        static thread_local size_t pinned_n = 0;
        static thread_local cudaStream_t ust = nullptr;
        static thread_local int ust_dev = -1;
        if (ust_dev != r->device) {
            if (ust) cudaStreamDestroy(ust);
            ust = nullptr;
            CUDA_TRY(cudaStreamCreateWithFlags(&ust, cudaStreamNonBlocking));
            ust_dev = r->device;
        }
        if (pinned_n < r->bytes) {
            if (pinned) cudaFreeHost(pinned);
            pinned = nullptr;
            pinned_n = 0;
            CUDA_TRY(cudaMallocHost(&pinned, r->bytes));
            pinned_n = r->bytes;
        }
        int rc = arena_alloc(r->device, r->bytes, &r->arena, ust);
        if (rc != MCS_OK) return rc;
        memcpy(pinned, r->staging.data(), r->bytes);
        CUDA_TRY(cudaMemcpyAsync(r->arena, pinned, r->bytes, cudaMemcpyHostToDevice, ust));
        CUDA_TRY(cudaStreamSynchronize(ust));
    }
    const uintptr_t base = (uintptr_t)r->arena;
    Rep &R = r->rep;
#define RELOC(f) if (R.f) R.f = (decltype(R.f))((uintptr_t)R.f + base)
    RELOC(nbr); RELOC(lcode); RELOC(lcls); RELOC(deg); RELOC(stype); RELOC(jtab); RELOC(jtab64); RELOC(dtab);
    RELOC(itab); RELOC(cpair); RELOC(rorb); RELOC(rcl); RELOC(rlink); RELOC(rjc); RELOC(rK); RELOC(rkc);
    RELOC(rdeg); RELOC(rindex); RELOC(circ); RELOC(slen); RELOC(sval); RELOC(gmask); RELOC(sflag); RELOC(rtgt);
    RELOC(spins); RELOC(acc); RELOC(series); RELOC(icnt); RELOC(stats); RELOC(wbits); RELOC(wqueue); RELOC(wmaj);
#undef RELOC
    if (const SharedLists *sh = r->shared) {
        R.nbr = sh->nbr; R.lcode = sh->lcode; R.deg = sh->deg; R.stype = sh->stype;
        R.cpair = sh->cpair; R.rorb = sh->rorb; R.rcl = sh->rcl; R.rlink = sh->rlink; R.rjc = sh->rjc;
        R.rdeg = sh->rdeg; R.rindex = sh->rindex; R.circ = sh->circ; R.slen = sh->slen; R.sval = sh->sval;
        R.gmask = sh->gmask; R.sflag = sh->sflag; R.rtgt = sh->rtgt;
    }
    // spin frames: kernels store each snapshot straight into page-locked host
    // memory mapped into the device, so frames take no device memory and need
    // no copy at the end
    if (r->frames_bytes > 0 && !r->frames_host) {
        CUDA_TRY(cudaHostAlloc(&r->frames_host, r->frames_bytes, cudaHostAllocMapped | cudaHostAllocPortable));
        void *dp = nullptr;
        CUDA_TRY(cudaHostGetDevicePointer(&dp, r->frames_host, 0));
        R.frame_buf = dp;
    }
    std::vector<unsigned char>().swap(r->staging);
    return MCS_OK;
}

// ------------------------------------------------------------------ results
int fetch_result_blocks(const std::vector<Replica *> &rs, int device)
{
    if (rs.empty()) return MCS_OK;
    CUDA_TRY(cudaSetDevice(device));
    static thread_local void *pinned = nullptr;
    static thread_local size_t pinned_n = 0;
    static thread_local cudaStream_t rst = nullptr;
    static thread_local int rst_dev = -1;
    if (rst_dev != device) {
        if (rst) cudaStreamDestroy(rst);
        rst = nullptr;
        CUDA_TRY(cudaStreamCreateWithFlags(&rst, cudaStreamNonBlocking));
        rst_dev = device;
    }
    size_t total = 0;
    std::vector<size_t> off(rs.size()), len(rs.size());
    for (size_t i = 0; i < rs.size(); ++i) {
        off[i] = total;
        len[i] = rs[i]->stats_off + S_NSTAT * sizeof(long long) - rs[i]->acc_off;
        total += (len[i] + 15) & ~(size_t)15;
    }
    if (pinned_n < total) {
        if (pinned) cudaFreeHost(pinned);
        pinned = nullptr;
        pinned_n = 0;
        CUDA_TRY(cudaMallocHost(&pinned, total));
        pinned_n = total;
    }
    for (size_t i = 0; i < rs.size(); ++i)
        CUDA_TRY(cudaMemcpyAsync((unsigned char *)pinned + off[i], (unsigned char *)rs[i]->arena + rs[i]->acc_off, len[i],
                                 cudaMemcpyDeviceToHost, rst));
    CUDA_TRY(cudaStreamSynchronize(rst));
    for (size_t i = 0; i < rs.size(); ++i) {
        rs[i]->rblock.assign((unsigned char *)pinned + off[i], (unsigned char *)pinned + off[i] + len[i]);
        rs[i]->rblock_fresh = true;
    }
    return MCS_OK;
}

int replica_results(Replica *r, const Rep &Rfinal, mcs_result *res)
{
    const HostModel &m = r->hm;
    std::vector<double> acc(r->nacc);
    std::vector<long long> icnt(C_NINT), stats(S_NSTAT);
    unsigned char *b = (unsigned char *)r->arena;
    if (!r->rblock_fresh) {
        int rc = fetch_result_blocks({r}, r->device);
        if (rc != MCS_OK) return rc;
    }
    {
        // the block spans acc .. stats in the arena (consecutive regions)
        const unsigned char *h = r->rblock.data();
        memcpy(acc.data(), h, acc.size() * sizeof(double));
        memcpy(icnt.data(), h + (r->icnt_off - r->acc_off), icnt.size() * sizeof(long long));
        memcpy(stats.data(), h + (r->stats_off - r->acc_off), stats.size() * sizeof(long long));
    }
    if (!res) return MCS_OK;
    double *g = res->group_values;
    int gcap = res->group_capacity;
    float *fr = res->frames;
    double *ser = res->series;
    memset(res->values, 0, sizeof res->values);
    const double ns = (double)m.nsweep, nl = (double)m.nlat;
    double *v = res->values;
    if (m.dim == 1) {
        double M2 = acc[B_M2], M4 = acc[B_M4], Mt = acc[B_MTOT];
        v[0] = acc[B_SI] / ns; v[1] = acc[B_SJ] / ns; v[2] = acc[B_SIJ] / ns;
        v[3] = (acc[B_MDM] / ns - (Mt / ns) * (Mt / ns));
        v[4] = acc[B_E] / ns; v[5] = acc[B_E2] / ns; v[6] = acc[B_ER] / ns; v[7] = acc[B_ER2] / ns;
        v[8] = (M2 / ns) * (M2 / ns) / (M4 / ns);
        v[9] = acc[B_STOT] / ns / nl;
    } else {
        bool xy = m.dim == 2;
        double M2 = acc[A_M2], M4 = acc[A_M4], Mt = acc[A_MTOT];
        v[0] = acc[A_SI] / ns; v[1] = acc[A_SI + 1] / ns; v[2] = xy ? 0 : acc[A_SI + 2] / ns;
        v[3] = acc[A_SJ] / ns; v[4] = acc[A_SJ + 1] / ns; v[5] = xy ? 0 : acc[A_SJ + 2] / ns;
        v[6] = acc[A_SIJ] / ns;
        v[7] = xy ? (acc[A_MDM] / ns - (Mt / ns) * (Mt / ns)) : (acc[A_MDM] / ns - Mt / ns * Mt / ns);
        v[8] = acc[A_E] / ns; v[9] = acc[A_E2] / ns;
        v[10] = (M2 / ns) * (M2 / ns) / (M4 / ns);
        v[11] = acc[A_SIR] / ns; v[12] = acc[A_SIR + 1] / ns; v[13] = xy ? 0 : acc[A_SIR + 2] / ns;
        v[14] = acc[A_SJR] / ns; v[15] = acc[A_SJR + 1] / ns; v[16] = xy ? 0 : acc[A_SJR + 2] / ns;
        v[17] = acc[A_SIJR] / ns; v[18] = acc[A_ER] / ns; v[19] = acc[A_ER2] / ns;
        v[20] = acc[A_SIZ] / ns; v[21] = acc[A_SJZ] / ns; v[22] = acc[A_STZ] / ns;
        v[23] = acc[A_SIH] / ns; v[24] = acc[A_SJH] / ns; v[25] = acc[A_STH] / ns;
        v[26] = xy ? 0 : acc[A_Q] / ns;
        int G = m.ngroup, ng = (G + 1) * (G + 1) + (G + 1);
        if (g && G > 0)
            for (int k = 0; k < ng && k < gcap; ++k) g[k] = acc[A_GRP + k] / ns;
        res->energy_drift = acc[A_DRIFT];
    }
    res->frames_written = 0;
    if (fr && m.frames > 0 && r->frames_host) {
        // the kernels stored the frames in sweep-index order (Ising: signs;
        // O(n): dim components); the reference's order and layout are site id
        // order with three components
        const int nf = std::min(Rfinal.frames_written, m.frames), N = m.N;
        for (int f = 0; f < nf; ++f) {
            float *o = fr + (size_t)f * N * 3;
            if (m.dim == 1) {
                const signed char *sb = (const signed char *)r->frames_host + (size_t)f * N;
                for (int i = 0; i < N; ++i) {
                    const int k = m.pos[i];
                    o[3 * i] = (float)(fabs(m.sval[k]) * sb[k]);
                    o[3 * i + 1] = 0.f;
                    o[3 * i + 2] = 0.f;
                }
            } else {
                const float *fb = (const float *)r->frames_host + (size_t)f * N * m.dim;
                for (int i = 0; i < N; ++i) {
                    const int k = m.pos[i];
                    for (int c = 0; c < 3; ++c) o[3 * i + c] = c < m.dim ? fb[(size_t)k * m.dim + c] : 0.f;
                }
            }
        }
        res->frames_written = nf;
    }
    if (ser && r->record_series)
        CUDA_TRY(cudaMemcpy(ser, b + r->series_off, (size_t)m.nsweep * MCS_NSER * sizeof(double), cudaMemcpyDeviceToHost));
    res->accepted = stats[S_ACCEPT];
    res->clusters = stats[S_CLUSTERS];
    res->flipped = stats[S_FLIPPED];
    res->site_updates = m.alg == 0 ? stats[S_VISITS] : stats[S_FLIPPED];
    res->exact_mismatches = m.dim == 1 ? icnt[C_MISM] : 0;
    res->n_colours = m.ncol;
    res->schedule_used = r->schedule;
    return MCS_OK;
}

int replica_spins(Replica *r, std::vector<double> &out)
{
    const HostModel &m = r->hm;
    out.assign((size_t)3 * m.N, 0.0);
    unsigned char *b = (unsigned char *)r->arena;
    if (m.dim == 1) {
        std::vector<int8_t> s(m.N);
        CUDA_TRY(cudaMemcpy(s.data(), b + r->spins_off, m.N, cudaMemcpyDeviceToHost));
        for (int i = 0; i < m.N; ++i) out[3 * i] = fabs(m.sval[m.pos[i]]) * s[m.pos[i]];
    } else {
        std::vector<float> s((size_t)m.dim * r->rep.spad);
        CUDA_TRY(cudaMemcpy(s.data(), b + r->spins_off, s.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (int i = 0; i < m.N; ++i)
            for (int c = 0; c < m.dim; ++c) out[3 * i + c] = s[(size_t)c * r->rep.spad + m.pos[i]];
    }
    return MCS_OK;
}

int replica_set_spins(Replica *r, const double *in)
{
    const HostModel &m = r->hm;
    unsigned char *b = (unsigned char *)r->arena;
    if (m.dim == 1) {
        std::vector<int8_t> s(m.N);
        for (int i = 0; i < m.N; ++i) s[m.pos[i]] = in[3 * i] < 0 ? -1 : 1;
        CUDA_TRY(cudaMemcpy(b + r->spins_off, s.data(), m.N, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> s((size_t)m.dim * r->rep.spad, 0.f);
        for (int i = 0; i < m.N; ++i)
            for (int c = 0; c < m.dim; ++c) s[(size_t)c * r->rep.spad + m.pos[i]] = (float)in[3 * i + c];
        CUDA_TRY(cudaMemcpy(b + r->spins_off, s.data(), s.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    return MCS_OK;
}

// ------------------------------------------------------------------ batch execution
Batch::~Batch()
{
    // work of this batch may still be queued (a prepared batch that never
    // advanced); the arenas are freed stream-ordered on the default stream
    if (stream) cudaStreamSynchronize(stream);
    for (cudaStream_t g : gstreams) cudaStreamSynchronize(g);
    for (cudaStream_t g : gstreams_hi) cudaStreamSynchronize(g);
    groups.clear();
    buf_free(d_reps);
    buf_free(d_stop);
    if (h_stop) cudaFreeHost(h_stop);
    buf_free(d_scratch);
    for (cudaEvent_t e : tev) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
    if (stream2) cudaStreamDestroy(stream2);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev_a) cudaEventDestroy(ev_a);
    if (ev_b) cudaEventDestroy(ev_b);
    if (ev_fork) cudaEventDestroy(ev_fork);
    for (cudaStream_t g : gstreams) cudaStreamDestroy(g);
    for (cudaStream_t g : gstreams_hi) cudaStreamDestroy(g);
    for (cudaEvent_t e : gevents) cudaEventDestroy(e);
}

int Batch::init(int dev)
{
    device = dev;
    return MCS_OK;
}

int Batch::ensure_streams()
{
    if (stream) return MCS_OK;
    CUDA_TRY(cudaSetDevice(device));
    CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&ev0));
    CUDA_TRY(cudaEventCreate(&ev1));
    CUDA_TRY(cudaEventCreate(&ev_a));
    CUDA_TRY(cudaEventCreate(&ev_b));
    CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    return MCS_OK;
}

int Batch::add(const mcs_problem *p, const mcs_options *o, int *idx)
{
    std::unique_ptr<Replica> r(new Replica());
    r->device = device;
    // O(n) replicas of a lattice already compiled in this batch (a grid of
    // temperatures and fields) take its structure from that replica's template
    std::shared_ptr<const ModelTemplate> t;
    const bool on = p && p->model != MCS_ISING;
    if (on) {
        std::lock_guard<std::mutex> lock(add_mutex);
        for (auto it = templates.rbegin(); it != templates.rend() && !t; ++it)
            if ((*it)->in.model == p->model && (*it)->in.N == p->n_sites && (*it)->in.z == p->max_links) t = *it;
    }
    // the index arrays of that lattice, uploaded once for the batch
    const SharedLists *sh = nullptr;
    if (t) {
        std::lock_guard<std::mutex> lock(add_mutex);
        auto it = shared_lists.find(t.get());
        if (it == shared_lists.end()) {
            std::unique_ptr<SharedLists> nsh;
            int rc = make_shared_lists(t->hm, device, &nsh);
            if (rc != MCS_OK) return rc;
            it = shared_lists.emplace(t.get(), std::move(nsh)).first;
        }
        sh = it->second.get();
    }
    bool reused = false;
    int rc = build_replica(p, o, r.get(), true, t.get(), &reused, sh);
    if (rc != MCS_OK) return rc;
    std::shared_ptr<const ModelTemplate> nt;
    if (on && !reused) {
        bool have = false;
        {
            std::lock_guard<std::mutex> lock(add_mutex);
            for (auto &q : templates) have |= q->in.model == p->model && q->in.N == p->n_sites && q->in.z == p->max_links;
            have |= templates.size() >= 8;
        }
        if (!have) nt = make_template(p, r->hm);
    }
    std::lock_guard<std::mutex> lock(add_mutex);
    if (prepared) { set_error("batch already prepared: add replicas before the first run or advance"); return MCS_EINVAL; }
    if (nt) templates.push_back(std::move(nt));
    replicas.push_back(std::move(r));
    if (idx) *idx = (int)replicas.size() - 1;
    return MCS_OK;
}

static int choose_schedule(const Replica &r, int requested, int max_smem)
{
    if (r.hm.alg == 1) {                     // Wolff: shared-memory or global state
        int g = 0;
        wolff_smem_bytes(r.rep, &g);
        return g ? 5 : 4;
    }
    if (requested == 1) return 1;            // plain
    if (requested == 3) return 3;            // tiled
    long long need = resident_smem_bytes(r.rep);
    if (requested == 2) return need <= max_smem ? 2 : 3;
    if (requested == 6 && r.hm.cluster_ok) return 6;
    if (need <= max_smem) return 2;
    if (r.hm.cluster_ok) return 6;
    return 3;
}

// ------------------------------------------------------------------ groups
// Replicas run in groups of one kernel family; each group is set up once
// (descriptor ids, tile lists, partial-sum buffers, captured graph) and then
// advanced by any number of units.
Group::~Group()
{
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void *p : bufs) buf_free(p);
    buf_free(d_ids);
}

int Batch::setup_tiled(Group &G)
{
    const int dim = G.dim, geom = G.geom;
    for (int id : G.ids) G.maxcol = std::max(G.maxcol, replicas[id]->hm.ncol);
    std::vector<std::vector<Item>> sweep(G.maxcol);
    const int per = dim == 1 ? 4 * 256 : 256;
    int slot = 0;
    std::vector<int> ioff(1, 0), moff(1, 0);
    std::vector<Item> meas;
    for (int id : G.ids) {
        const HostModel &m = replicas[id]->hm;
        for (int c = 0; c < m.ncol; ++c) {
            int n = m.col_start[c + 1] - m.col_start[c];
            for (int b0 = 0; b0 < n; b0 += per) {
                Item it; it.rep = id; it.begin = b0; it.end = std::min(n, b0 + per); it.slot = slot++;
                sweep[c].push_back(it);
            }
        }
        ioff.push_back(slot);
        // measurement tiles: the Ising frame's gathers are latency-bound, so
        // its tiles are smaller (one index per thread; 26.5 against 30.9 us
        // per sweep at L = 232)
        const int V = std::max(std::max(m.N, m.nlat), std::max(m.n_rorb, m.ncirc)), mt = dim == 1 ? 256 : 512;
        for (int b0 = 0; b0 < V; b0 += mt) {
            Item it; it.rep = id; it.begin = b0; it.end = std::min(V, b0 + mt); it.slot = 0;
            meas.push_back(it);
        }
        moff.push_back((int)meas.size());
    }
    std::vector<Item> all;
    for (auto &v : sweep) { G.cofs.push_back(all.size()); G.ccount.push_back((int)v.size()); all.insert(all.end(), v.begin(), v.end()); }
    G.nmeas = (int)meas.size();
    auto dalloc = [&](size_t bytes, void **p) -> int {
        CUDA_TRY(buf_alloc(device, p, bytes));
        G.bufs.push_back(*p);
        return MCS_OK;
    };
    int rc;
    if ((rc = dalloc(all.size() * sizeof(Item), (void **)&G.d_sw))) return rc;
    if ((rc = dalloc(meas.size() * sizeof(Item), (void **)&G.d_mi))) return rc;
    if ((rc = dalloc(ioff.size() * sizeof(int), (void **)&G.d_ioff))) return rc;
    if ((rc = dalloc(moff.size() * sizeof(int), (void **)&G.d_moff))) return rc;
    if ((rc = dalloc(std::max(1, slot) * sizeof(double), (void **)&G.d_dE))) return rc;
    if ((rc = dalloc(std::max(1, slot) * 9 * sizeof(long long), (void **)&G.d_ip))) return rc;
    if ((rc = dalloc(meas.size() * F_NON * sizeof(double), (void **)&G.d_fp))) return rc;
    CUDA_TRY(cudaMemcpy(G.d_sw, all.data(), all.size() * sizeof(Item), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(G.d_mi, meas.data(), meas.size() * sizeof(Item), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(G.d_ioff, ioff.data(), ioff.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(G.d_moff, moff.data(), moff.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(G.d_dE, 0, std::max(1, slot) * sizeof(double)));
    CUDA_TRY(cudaMemset(G.d_ip, 0, std::max(1, slot) * 9 * sizeof(long long)));
    (void)geom;
    return MCS_OK;
}

cudaError_t Batch::launch_group(Group &G, int C, int threads, long long units, cudaStream_t s)
{
    // C = 0: the resident kernel; C < 0: the resident kernel with -C copies of
    // each replica in a cluster; C >= 1: the row-split cluster kernel
    if (C <= 0)
        return launch_resident_metro(G.dim, G.geom, d_reps, G.d_ids, (int)G.ids.size(), threads, G.smem, units, s,
                                     C < 0 ? -C : 1);
    size_t sm = 0;
    for (int id : G.ids) sm = std::max<size_t>(sm, (size_t)cluster_smem_bytes(replicas[id]->rep, C));
    return launch_cluster_metro(G.dim, d_reps, G.d_ids, (int)G.ids.size(), C, threads, sm, units, s);
}

cudaError_t Batch::tiled_unit(Group &G, cudaStream_t s, long long *nl)
{
    for (int c = 0; c < G.maxcol; ++c) {
        cudaError_t e = launch_tiled_sweep(G.dim, G.geom, d_reps, G.d_sw + G.cofs[c], G.ccount[c], c, G.d_dE, G.d_ip, 256, s);
        if (e != cudaSuccess) return e;
        ++*nl;
    }
    cudaError_t e = launch_tiled_measure(G.dim, G.geom, d_reps, G.d_mi, G.nmeas, G.d_fp, 256, s);
    if (e != cudaSuccess) return e;
    e = launch_tiled_finalize_dim(G.dim, d_reps, G.d_ids, (int)G.ids.size(), G.d_ioff, G.d_dE, G.d_ip, G.d_moff, G.d_fp, s);
    *nl += 2;
    return e;
}

// Load balancing.  A launch of the resident kernel lasts as long as its
// largest replica (one CTA each), so one big replica among small ones leaves
// most SMs idle.  The balancer estimates the device time of a placement as
//     max( longest per-replica critical path, total SM-seconds / #SMs )
// with, per replica of c site updates,
//     resident:   critical c / r_cta,            SM-seconds c / r_cta
//     cluster C:  critical c / (e C r_cta),      SM-seconds c / (e r_cta)
//     tiled:      critical 0,                    SM-seconds c #SMs / r_dev(S)
// (r_cta = one CTA's rate, e = cluster efficiency, r_dev(S) = the tiled
// schedule's whole-device rate for S sites in flight, r_max S / (S + S_half):
// short launches are latency-bound; rates measured on GB300 for square
// lattices), and
// moves the replicas on the critical path one step (resident -> cluster 2 ->
// 4 -> 8 -> tiled; resident -> tiled where the cluster kernel does not apply)
// while the estimate falls.  With the autotuner on, cluster sizes stay the
// autotuner's choice and only the move to tiled is decided here.
void Batch::place_replicas(int max_smem, const std::vector<int> &ids, double base_crit, double base_smsec,
                           double base_ctas)
{
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || nsm < 1) {
        cudaGetLastError();
        nsm = 1;
    }
    static const double r_cta[4] = {0, 0.40e9, 0.85e9, 0.65e9};   // by spin dimension
    static const double r_max[4] = {0, 2.5e10, 1.8e10, 0.86e10};
    static const double s_half[4] = {0, 6.0e5, 1.0e6, 5.3e5};
    const double e = 0.8;
    struct P { int i; int opt; double c; std::vector<int> opts; };
    std::vector<P> ps;
    for (int i : ids) {
        Replica &r = *replicas[i];
        r.pref_C = 0;
        if (r.requested_schedule != 0 || r.hm.alg != 0 || !(r.schedule == 2 || r.schedule == 6)) continue;
        P q;
        q.i = i;
        q.c = (double)r.hm.N * (double)std::max<long long>(1, r.hm.units_total - r.rep.u);
        // options in order: 1 = resident, 2/4/8 = cluster, 0 = tiled
        const bool clusterable = r.hm.cluster_ok && r.hm.geom == MCS_GEOM_SQUARE && cluster_override != 1;
        if (clusterable && !no_autotune) {
            // the autotuner picks its cluster size; counted here as a cluster of 4
            q.opts.push_back(-1);
            q.opt = 0;
            ps.push_back(q);
            continue;
        }
        if (resident_smem_bytes(r.rep) <= max_smem) q.opts.push_back(1);
        if (clusterable)
            for (int C : {2, 4, 8, 16}) {
                if (r.hm.Lx / 2 < C || cluster_smem_bytes(r.rep, C) > max_smem) continue;
                if (cluster_override > 1 && C != cluster_override) continue;
                q.opts.push_back(C);
            }
        if (r.hm.N >= 8192 || q.opts.empty()) q.opts.push_back(0);
        q.opt = 0;
        ps.push_back(q);
    }
    if (ps.empty()) return;
    auto crit = [&](const P &q) {
        const int o = q.opts[q.opt], d = replicas[q.i]->hm.dim;
        if (o < 0) return q.c / (e * 4 * r_cta[d]);
        return o == 0 ? 0.0 : (o == 1 ? q.c / r_cta[d] : q.c / (e * o * r_cta[d]));
    };
    double tiled_sites[4] = {0, 0, 0, 0};
    auto smsec = [&](const P &q) {
        const int o = q.opts[q.opt], d = replicas[q.i]->hm.dim;
        if (o < 0) return q.c / (e * r_cta[d]);
        if (o == 0) {
            const double S = std::max(1.0, tiled_sites[d]);
            return q.c * nsm / (r_max[d] * S / (S + s_half[d]));
        }
        return o == 1 ? q.c / r_cta[d] : q.c / (e * r_cta[d]);
    };
    auto estimate = [&]() {
        for (int d = 0; d < 4; ++d) tiled_sites[d] = 0;
        for (auto &q : ps)
            if (q.opts[q.opt] == 0) tiled_sites[replicas[q.i]->hm.dim] += replicas[q.i]->hm.N;
        double m = base_crit, t = base_smsec;
        for (auto &q : ps) { m = std::max(m, crit(q)); t += smsec(q); }
        return std::max(m, t / nsm);
    };
    double best = estimate();
    for (int it = 0; it < 64; ++it) {
        double m = 0;
        for (auto &q : ps) m = std::max(m, crit(q));
        if (m <= 0) break;
        std::vector<int> moved;
        bool stuck = false;
        for (int k = 0; k < (int)ps.size(); ++k) {
            P &q = ps[k];
            if (crit(q) < 0.95 * m) continue;
            if (q.opt + 1 >= (int)q.opts.size()) { stuck = true; break; }
            ++q.opt;
            moved.push_back(k);
        }
        const double now = stuck ? best + 1 : estimate();
        if (now < best) { best = now; continue; }
        for (int k : moved) --ps[k].opt;
        break;
    }
    // Then, one replica at a time in order of its own critical path, a larger
    // cluster for any replica whose move does not lengthen the estimate: a
    // replica that cannot move (a lattice the cluster schedule cannot split) no
    // longer holds the others at one CTA, and each finishes as early as the
    // device allows.  Moves to the tiled schedule are left to the first pass.
    // The CTAs of all replicas (a resident or cluster CTA counted as one SM's
    // worth) stay within the device's SMs, and a slab keeps at least 8 rows:
    // beyond either, a larger cluster adds waves or barrier-bound CTAs instead
    // of speed.
    std::vector<char> frozen(ps.size(), 0);
    auto ctas = [&](const P &q) { const int o = q.opts[q.opt]; return o == 0 ? 0 : (o < 0 ? 4 : o); };
    double used = base_ctas;
    for (auto &q : ps) used += ctas(q);
    for (size_t it = 0; it < 4 * ps.size() + 4; ++it) {
        int pick = -1;
        double mc = 0;
        for (int k = 0; k < (int)ps.size(); ++k) {
            const P &q = ps[k];
            if (frozen[k] || q.opt + 1 >= (int)q.opts.size() || q.opts[q.opt + 1] <= 1) continue;
            const int nxt = q.opts[q.opt + 1];
            if (replicas[q.i]->hm.Lx / nxt < 8 || used - ctas(q) + nxt > nsm) continue;
            const double c = crit(q);
            if (c > mc) { mc = c; pick = k; }
        }
        if (pick < 0) break;
        used -= ctas(ps[pick]);
        ++ps[pick].opt;
        used += ctas(ps[pick]);
        const double now = estimate();
        if (now <= best * (1.0 + 1e-9)) best = std::min(best, now);
        else {
            used -= ctas(ps[pick]);
            --ps[pick].opt;
            used += ctas(ps[pick]);
            frozen[pick] = 1;
        }
    }
    for (auto &q : ps) {
        Replica &r = *replicas[q.i];
        const int o = q.opts[q.opt];
        if (o < 0) continue;
        if (o == 0) r.schedule = 3;
        else if (o == 1) r.schedule = 2;
        else if (no_autotune) { r.schedule = 6; r.pref_C = o; }
    }
}

// Kernel family of each replica of `ids` (and, with the balancer on, the
// placement among resident, cluster and tiled schedules).
void Batch::assign_schedules(const std::vector<int> &ids, int max_smem)
{
    for (int i : ids) {
        Replica &r = *replicas[i];
        r.schedule = choose_schedule(r, cluster_override > 1 ? 6 : r.requested_schedule, max_smem);
    }
    if (!balance) return;
    // replicas already running (slot mode) count as load the new ones share the
    // device with: their longest remaining critical path and SM-seconds on
    // their schedules (rates as in place_replicas)
    static const double r_cta[4] = {0, 0.40e9, 0.85e9, 0.65e9};
    std::vector<char> is_new(replicas.size(), 0);
    for (int i : ids) is_new[i] = 1;
    double base_crit = 0, base_smsec = 0, base_ctas = 0;
    for (size_t i = 0; i < replicas.size(); ++i) {
        const Replica *r = replicas[i].get();
        if (!r || is_new[i]) continue;
        const double c = (double)r->hm.N * (double)std::max<long long>(0, r->hm.units_total - r->rep.u);
        const double rc = r_cta[r->hm.dim];
        if (r->schedule == 6) {
            base_crit = std::max(base_crit, c / (0.8 * std::max(1, r->pref_C) * rc));
            base_smsec += c / (0.8 * rc);
            base_ctas += std::max(1, r->pref_C);
        } else if (r->schedule == 3) {
            base_smsec += c / (0.8 * rc);
        } else {
            base_crit = std::max(base_crit, c / rc);
            base_smsec += c / rc;
            base_ctas += 1;
        }
    }
    place_replicas(max_smem, ids, base_crit, base_smsec, base_ctas);
}

// Initial energies / exact sums (and random initial states) of the replicas of
// `ids` not yet initialised; their descriptors are on the device.
int Batch::init_states(const std::vector<int> &ids)
{
    std::vector<int> all;
    for (int i : ids)
        if (!replicas[i]->initialized) all.push_back(i);
    if (all.empty()) return MCS_OK;
    int *d = nullptr;
    CUDA_TRY(cudaMallocAsync((void **)&d, all.size() * sizeof(int), stream));
    CUDA_TRY(cudaMemcpyAsync(d, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
    for (int dd = 1; dd <= 3; ++dd)
        for (int g = 0; g <= 1; ++g) {
            bool any = false;
            for (int i : all) any |= (replicas[i]->hm.dim == dd && replicas[i]->hm.geom == g);
            if (!any) continue;
            cudaError_t e = launch_init_state_dg(dd, g, d_reps, d, (int)all.size(), stream);
            if (e != cudaSuccess) {
                cudaFreeAsync(d, stream);
                set_error(std::string("initial state: ") + cudaGetErrorString(e));
                return MCS_ECUDA;
            }
            launches++;
        }
    CUDA_TRY(cudaFreeAsync(d, stream));
    for (int i : all) replicas[i]->initialized = true;
    return MCS_OK;
}

// Device copy of a group's replica indices (reallocated when it grows).
int Batch::upload_ids(Group &G)
{
    if ((int)G.ids.size() > G.ids_cap) {
        buf_free(G.d_ids);
        G.d_ids = nullptr;
        G.ids_cap = 0;
        const int cap = std::max<int>(4, (int)G.ids.size() * 2);
        CUDA_TRY(buf_alloc(device, (void **)&G.d_ids, cap * sizeof(int)));
        G.ids_cap = cap;
    }
    if (!G.ids.empty())
        CUDA_TRY(cudaMemcpy(G.d_ids, G.ids.data(), G.ids.size() * sizeof(int), cudaMemcpyHostToDevice));
    return MCS_OK;
}

// A tiled group whose membership changed: new tile lists, partial-sum
// buffers and graph.
int Batch::reset_tiled(Group &G)
{
    if (G.exec) cudaGraphExecDestroy(G.exec);
    if (G.graph) cudaGraphDestroy(G.graph);
    G.exec = nullptr;
    G.graph = nullptr;
    for (void *q : G.bufs) buf_free(q);
    G.bufs.clear();
    G.cofs.clear();
    G.ccount.clear();
    G.maxcol = 0;
    G.nmeas = 0;
    G.K = 0;
    G.per_graph = 0;
    return setup_tiled(G);
}

// Groups for the replicas of `ids` (each joins exactly one; a cluster group
// that falls back to the tiled schedule keeps its replicas).  With `merge`,
// a set whose launch configuration equals that of an existing group joins it
// instead of forming a new one (the server admits a few requests at a time).
int Batch::build_groups(const std::vector<int> &ids, bool merge)
{
    const int max_smem = resident_max_smem();
    int nsm_ = 0;
    if (cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        nsm_ = 1;
    }
    std::vector<char> grouped(replicas.size(), 0);
    for (int kind : {2, 6, 3, 1, 4, 5})
        for (int d = 1; d <= 3; ++d)
            for (int g = 0; g <= 1; ++g) {
                std::vector<int> sel;
                for (int i : ids) {
                    Replica &r = *replicas[i];
                    if (!grouped[i] && r.schedule == kind && r.hm.dim == d && r.hm.geom == g) sel.push_back(i);
                }
                for (int i : sel) grouped[i] = 1;
                if (sel.empty()) continue;
                std::vector<std::vector<int>> sets;
                if (kind == 1) for (int id : sel) sets.push_back({id});
                else if (kind == 6) {
                    // one launch configuration per group: split by the balancer's cluster size
                    for (int C : {0, 2, 4, 8, 16}) {
                        std::vector<int> sub;
                        for (int id : sel) if (replicas[id]->pref_C == C) sub.push_back(id);
                        if (!sub.empty()) sets.push_back(sub);
                    }
                } else if (kind == 2 && slot_capacity > 0) {
                    // a server's resident replicas by size (factors of 4 in sites): a
                    // group's quotas follow its slowest member's measured pace, so a
                    // small lattice grouped with a large one would advance at the
                    // large one's speed
                    std::map<int, std::vector<int>> by;
                    for (int id : sel) {
                        int b = 0;
                        for (long long n = replicas[id]->hm.N; n > 4; n >>= 2) ++b;
                        by[b].push_back(id);
                    }
                    for (auto &kv : by) sets.push_back(kv.second);
                } else sets.push_back(sel);
                for (auto &set : sets) {
                    std::unique_ptr<Group> G(new Group());
                    G->kind = kind; G->dim = d; G->geom = g; G->ids = set;
                    long long maxn = 0;
                    int maxcs = 0;
                    for (int id : set) {
                        Replica &r = *replicas[id];
                        G->max_units = std::max(G->max_units, r.hm.units_total - r.rep.u);
                        maxn = std::max<long long>(maxn, r.hm.N);
                        G->smem = std::max<size_t>(G->smem, (size_t)resident_smem_bytes(r.rep));
                        for (int c = 0; c < r.hm.ncol; ++c)
                            maxcs = std::max(maxcs, r.hm.col_start[c + 1] - r.hm.col_start[c]);
                    }
                    if (kind == 4 || kind == 5) {
                        int gs = 0;
                        G->smem = 0;
                        for (int id : set) G->smem = std::max<size_t>(G->smem, (size_t)wolff_smem_bytes(replicas[id]->rep, &gs));
                        G->threads = threads_override > 0 ? threads_override : 512;
                        G->chunk = 1 << 20;
                        if (chunk_override > 0) G->chunk = chunk_override;
                    } else if (kind == 2 || kind == 6) {
                        int work = d == 1 ? (maxcs + 3) / 4 : maxcs;
                        G->threads = std::min(1024, std::max(64, ((work + 31) / 32) * 32));
                        if (threads_override > 0) G->threads = threads_override;
                        G->chunk = std::max<long long>(1, (1LL << 28) / std::max<long long>(1, maxn));
                        if (chunk_override > 0) G->chunk = chunk_override;
                        // candidate configurations for the autotuner: the resident
                        // kernel (C = 0), and every cluster size that divides each
                        // replica's rows into even slabs that fit in shared memory
                        // (C = 1: the cluster kernel on one CTA, whose measurement
                        // needs no index lists on regular lattices)
                        bool all_cl = g == MCS_GEOM_SQUARE;
                        for (int id : set) all_cl &= replicas[id]->hm.cluster_ok != 0;
                        int copies_only = 0;  // MCSGPU_COPIES=k: only the resident kernel with k copies
                        if (const char *e = getenv("MCSGPU_COPIES")) copies_only = atoi(e);
                        if (kind == 2 && copies_only > 1) {
                            if (resident_copies_active(d, g, copies_only, G->threads, G->smem) > 0)
                                G->candidates.push_back({-copies_only, G->threads});
                            else
                                G->candidates.push_back({0, G->threads});
                        } else if (kind == 2) {
                            G->candidates.push_back({0, G->threads});
                            // one warp per replica (a CTA of 32 threads): for groups of many
                            // small replicas that fill the device anyway, where the barriers
                            // and block reductions of a larger CTA cost more than its threads
                            // gain; the autotuner keeps it only where it is faster
                            if ((int)set.size() >= 32 && G->threads > 32) G->candidates.push_back({0, 32});
                            // copies of each replica over a cluster of 2 or 4 CTAs: for groups
                            // that would leave SMs idle (Metropolis only)
                            bool metro = true;
                            for (int id : set) metro &= replicas[id]->hm.alg == 0;
                            for (int cp : {2, 4})
                                if (metro && cluster_override != 1 && (int)set.size() * cp <= 2 * nsm_ &&
                                    resident_copies_active(d, g, cp, G->threads, G->smem) > 0)
                                    G->candidates.push_back({-cp, G->threads});
                        }
                        if (all_cl && cluster_override != 1 && copies_only <= 1) {
                            const int pc = kind == 6 ? replicas[set[0]]->pref_C : 0;
                            for (int C : {1, 2, 4, 8, 16}) {
                                if (C == 1 && kind != 2) continue;
                                if (cluster_override > 1 && C != cluster_override) continue;
                                if (pc > 0 && C != pc) continue;
                                // a group of small lattices that fills the device on one CTA
                                // each gains nothing from splitting them (more waves, and a
                                // slab of a few rows is all ghost rows): it is not probed on
                                // clusters of 2 or more
                                if (C >= 2 && pc == 0 && cluster_override <= 1 && (int)set.size() >= nsm_) {
                                    long long maxn = 0;
                                    for (int id : set) maxn = std::max<long long>(maxn, replicas[id]->hm.N);
                                    if (maxn <= 4096) continue;
                                }
                                bool ok = true;
                                size_t sm = 0;
                                for (int id : set) {
                                    // every CTA holds at least one row pair
                                    ok &= replicas[id]->hm.Lx / 2 >= C;
                                    sm = std::max<size_t>(sm, (size_t)cluster_smem_bytes(replicas[id]->rep, C));
                                }
                                if (!ok || (int)sm > max_smem) continue;
                                for (int th : {512, 256, 1024})
                                    if (cluster_active(d, C, th, sm) > 0) G->candidates.push_back({C, th});
                            }
                            // a wave-filling size: the largest cluster size at which every
                            // replica of the group runs at once, when it lies above the
                            // largest such power of two (32 replicas at 2 CTAs per SM on 152
                            // SMs: 9 CTAs each, 288 CTAs, beside 8 CTAs each, 256 CTAs)
                            auto fits = [&](int C, int th) {
                                size_t sm = 0;
                                for (int id : set) {
                                    if (replicas[id]->hm.Lx / 2 < C) return false;
                                    sm = std::max<size_t>(sm, (size_t)cluster_smem_bytes(replicas[id]->rep, C));
                                }
                                return (int)sm <= max_smem && cluster_active(d, C, th, sm) >= (int)set.size();
                            };
                            if (cluster_override <= 1 && pc == 0)
                                for (int th : {512, 256, 1024}) {
                                    int top = 0;
                                    for (const auto &c : G->candidates)
                                        if (c.second == th && c.first > top && fits(c.first, th)) top = c.first;
                                    if (getenv("MCSGPU_TRACE")) {
                                        fprintf(stderr, "mcsgpu trace: %zu replicas, %d threads, clusters at once by size:", set.size(), th);
                                        for (int C = 2; C <= 16; ++C) {
                                            size_t sm = 0;
                                            for (int id : set) sm = std::max<size_t>(sm, (size_t)cluster_smem_bytes(replicas[id]->rep, C));
                                            fprintf(stderr, " %d:%d", C, (int)sm <= max_smem ? cluster_active(d, C, th, sm) : 0);
                                        }
                                        fprintf(stderr, "\n");
                                    }
                                    if (top == 0) continue;
                                    for (int C = 16; C > top; --C)
                                        if ((C & (C - 1)) != 0 && fits(C, th)) {
                                            G->candidates.push_back({C, th});
                                            break;
                                        }
                                }
                            G->can_cluster = 1;
                        }
                        if (G->candidates.empty() && kind == 6) {
                            // no cluster size fits: run these replicas on the tiled schedule
                            G->kind = 3;
                            for (int id : set) replicas[id]->schedule = 3;
                        } else {
                            if (G->candidates.empty()) G->candidates.push_back({0, G->threads});
                            // MCSGPU_FORCE=C:threads keeps only that candidate when the group has it
                            // (tests run every configuration of a group this way)
                            if (const char *e = getenv("MCSGPU_FORCE")) {
                                int fc = 0, ft = 0;
                                if (sscanf(e, "%d:%d", &fc, &ft) == 2)
                                    for (auto &cand : G->candidates)
                                        if (cand.first == fc && cand.second == ft) { G->candidates = {cand}; break; }
                            }
                            if (G->candidates.size() == 1 || no_autotune) {
                                // without the autotuner: the first candidate, except that a
                                // resident group runs the one-CTA cluster kernel when it can
                                size_t pick = 0;
                                for (size_t ci = 0; ci < G->candidates.size() && kind == 2; ++ci)
                                    if (G->candidates[ci].first == 1) { pick = ci; break; }
                                G->C = G->candidates[pick].first;
                                G->threads = G->candidates[pick].second;
                                G->tuned = 1;
                            }
                        }
                    }
                    if (merge) {
                        // an existing group of the same launch configuration takes the set
                        Group *H = nullptr;
                        auto size_bucket = [&](const std::vector<int> &ids_) {
                            long long mx = 0;
                            for (int id : ids_) mx = std::max<long long>(mx, replicas[id]->hm.N);
                            int b = 0;
                            for (long long n = mx; n > 4; n >>= 2) ++b;
                            return b;
                        };
                        for (auto &q : groups) {
                            if (q->kind != G->kind || q->dim != d || q->geom != g || q->kind == 1) continue;
                            if (q->kind == 2 || q->kind == 6) {
                                if (!q->tuned || !G->tuned || q->C != G->C || q->threads != G->threads) continue;
                            }
                            if (q->kind == 2 && slot_capacity > 0 && size_bucket(q->ids) != size_bucket(G->ids)) continue;
                            H = q.get();
                            break;
                        }
                        if (H) {
                            H->ids.insert(H->ids.end(), set.begin(), set.end());
                            H->max_units = std::max(H->max_units, G->max_units);
                            H->smem = std::max(H->smem, G->smem);
                            H->chunk = std::min(H->chunk, G->chunk);
                            int rc = upload_ids(*H);
                            if (rc == MCS_OK && (H->kind == 3 || H->kind == 1)) rc = reset_tiled(*H);
                            if (rc != MCS_OK) return rc;
                            continue;
                        }
                    }
                    int rc = upload_ids(*G);
                    if (rc != MCS_OK) return rc;
                    if (G->kind == 3 || G->kind == 1) {
                        rc = setup_tiled(*G);
                        if (rc != MCS_OK) return rc;
                    }
                    groups.push_back(std::move(G));
                }
            }
    for (int i : ids)
        if (!grouped[i]) { set_error("internal: replica without a kernel group"); return MCS_EINVAL; }
    return MCS_OK;
}

int Batch::setup_device()
{
    cudaGetLastError();  // a failed call of an earlier batch must not be reported here
    int src = ensure_streams();
    if (src != MCS_OK) return src;
    if (const char *e = getenv("MCSGPU_CLUSTER")) cluster_override = atoi(e);
    if (const char *e = getenv("MCSGPU_NO_AUTOTUNE")) no_autotune = atoi(e);
    return MCS_OK;
}

int Batch::prepare()
{
    if (prepared) return MCS_OK;
    int rc = setup_device();
    if (rc != MCS_OK) return rc;
    const int nrep = (int)replicas.size();
    if (nrep == 0) { prepared = true; return MCS_OK; }
    std::vector<int> ids(nrep);
    for (int i = 0; i < nrep; ++i) ids[i] = i;
    assign_schedules(ids, resident_max_smem());
    std::vector<Rep> host(nrep);
    for (int i = 0; i < nrep; ++i) host[i] = replicas[i]->rep;
    CUDA_TRY(buf_alloc(device, (void **)&d_reps, nrep * sizeof(Rep)));
    CUDA_TRY(cudaMemcpy(d_reps, host.data(), nrep * sizeof(Rep), cudaMemcpyHostToDevice));
    rc = init_states(ids);
    if (rc != MCS_OK) return rc;
    rc = build_groups(ids, false);
    if (rc != MCS_OK) return rc;
    prepared = true;
    return MCS_OK;
}

// ------------------------------------------------------------------ slots (server)
// The server keeps one batch whose replicas vector is indexed by slot (null =
// free).  Replicas join and leave between steps; only the groups they join or
// leave change, and each replica advances by its own quota per step.
int Batch::admit(const std::vector<int> &ids, double step_us)
{
    if (ids.empty()) return MCS_OK;
    if (!d_reps) {
        int rc = setup_device();
        if (rc != MCS_OK) return rc;
        CUDA_TRY(buf_alloc(device, (void **)&d_reps, (size_t)slot_capacity * sizeof(Rep)));
        prepared = true;
    }
    const int max_smem = resident_max_smem();
    assign_schedules(ids, max_smem);
    // quota: the units a replica advances per step, so that each replica's
    // share of a step takes about step_us of device time on its schedule
    set_quotas(ids, step_us);
    for (int i : ids) replicas[i]->rep.u_stop = replicas[i]->rep.u;  // nothing runs before the step sets its bound
    for (int i : ids) CUDA_TRY(cudaMemcpyAsync(d_reps + i, &replicas[i]->rep, sizeof(Rep), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    int rc = init_states(ids);
    if (rc != MCS_OK) return rc;
    return build_groups(ids, true);
}

// Placement of the replicas that remain after others left: the balancer runs
// again over every active replica (with no other load), and a replica whose
// schedule or cluster size changes moves to the group of its new
// configuration (its state is in its arena between launches, so a move needs
// no copy).  Its quota restarts from the estimate of the new schedule.
int Batch::rebalance(double step_us, std::vector<int> *orphans)
{
    std::vector<int> ids;
    for (size_t i = 0; i < replicas.size(); ++i)
        if (replicas[i]) ids.push_back((int)i);
    if (ids.empty() || !balance) return MCS_OK;
    std::vector<std::pair<int, int>> before;
    for (int i : ids) before.push_back({replicas[i]->schedule, replicas[i]->pref_C});
    assign_schedules(ids, resident_max_smem());
    std::vector<int> moved;
    for (size_t k = 0; k < ids.size(); ++k) {
        Replica &r = *replicas[ids[k]];
        if (r.schedule != before[k].first || r.pref_C != before[k].second) moved.push_back(ids[k]);
    }
    if (getenv("MCSGPU_TRACE")) {
        fprintf(stderr, "mcsgpu trace: rebalance %zu active, %zu moved:", ids.size(), moved.size());
        for (int i : ids)
            fprintf(stderr, " [%d N=%d sched %d C %d]", i, replicas[i]->hm.N, replicas[i]->schedule, replicas[i]->pref_C);
        fprintf(stderr, "\n");
    }
    if (moved.empty()) return MCS_OK;
    drop(moved, orphans);
    set_quotas(moved, step_us);
    return build_groups(moved, true);
}

// Initial quota of the replicas of `ids` from their schedule: the units that
// take about step_us on it (measured rates per CTA: resident 1, cluster C:
// about 0.8 C, tiled about 4); the measured group times then adjust it.
void Batch::set_quotas(const std::vector<int> &ids, double step_us)
{
    static const double r_cta[4] = {0, 0.40e9, 0.85e9, 0.65e9};
    quota_ms = step_us * 1e-3;
    for (int i : ids) {
        Replica &r = *replicas[i];
        double ctas = 1.0;
        if (r.schedule == 6) ctas = 0.8 * std::max(1, r.pref_C);
        else if (r.schedule == 3) ctas = 4.0;
        const double per_unit = (double)r.hm.N / (r_cta[r.hm.dim] * ctas);
        const long long q = (long long)(step_us * 1e-6 / per_unit);
        r.rep.quota = std::max(1LL, std::min(q, r.hm.units_total));
    }
}

// Take the replicas of `ids` out of their groups.  A group whose device lists
// cannot be rebuilt is dissolved and its other replicas are returned in
// *orphans (the caller fails them).
void Batch::drop(const std::vector<int> &ids, std::vector<int> *orphans)
{
    if (ids.empty()) return;
    std::vector<char> gone(replicas.size(), 0);
    for (int i : ids) gone[i] = 1;
    for (auto &G : groups) {
        const size_t n0 = G->ids.size();
        G->ids.erase(std::remove_if(G->ids.begin(), G->ids.end(), [&](int i) { return gone[i] != 0; }), G->ids.end());
        if (G->ids.size() == n0 || G->ids.empty()) continue;
        if (upload_ids(*G) != MCS_OK || ((G->kind == 3 || G->kind == 1) && reset_tiled(*G) != MCS_OK)) {
            cudaGetLastError();
            if (orphans) orphans->insert(orphans->end(), G->ids.begin(), G->ids.end());
            G->ids.clear();
        }
    }
    groups.erase(std::remove_if(groups.begin(), groups.end(), [](const std::unique_ptr<Group> &G) { return G->ids.empty(); }),
                 groups.end());
}

// Autotuner results kept for the life of the process, keyed by the group's
// shape (kind, model dimension, geometry, replica count and sizes, coupling
// flags, measurement interval) and its candidate list, so that a batch of the
// same shape -- the next request of a sweep over (T, H) grids, the next bench
// step -- starts with the configuration found before instead of probing again.
static std::mutex g_tune_mutex;
static std::map<std::string, std::pair<int, int>> g_tune_cache;

static std::string tune_key(const Batch &b, const Group &G)
{
    long long sumn = 0, maxn = 0, upm_lo = 1LL << 62, upm_hi = 0;
    int flags = 0;
    for (int id : G.ids) {
        const Replica &r = *b.replicas[id];
        sumn += r.hm.N;
        maxn = std::max<long long>(maxn, r.hm.N);
        upm_lo = std::min<long long>(upm_lo, r.hm.upm);
        upm_hi = std::max<long long>(upm_hi, r.hm.upm);
        flags |= (r.rep.fullJ ? 1 : 0) | (r.rep.has_d ? 2 : 0) | (r.hm.ncirc > 0 ? 4 : 0) | (r.hm.meas_regular ? 8 : 0) |
                 (r.hm.ngroup > 0 ? 16 : 0);
    }
    std::string k = std::to_string(G.kind) + "/" + std::to_string(G.dim) + "/" + std::to_string(G.geom) + "/" +
                    std::to_string(G.ids.size()) + "/" + std::to_string(sumn) + "/" + std::to_string(maxn) + "/" +
                    std::to_string(upm_lo) + "-" + std::to_string(upm_hi) + "/" + std::to_string(flags) + "/";
    for (auto &c : G.candidates) k += std::to_string(c.first) + "x" + std::to_string(c.second) + ",";
    return k;
}

int Batch::advance(long long units)
{
    int rc = prepare();
    if (rc != MCS_OK) return rc;
    if (replicas.empty()) return MCS_OK;
    for (auto &r : replicas) r->rblock_fresh = false;
    CUDA_TRY(cudaEventRecord(ev0, stream));
    // 1. autotuner: time each candidate (cluster size, block size) of an
    //    untuned group on a few real units, alone on the batch stream, and keep
    //    the fastest
    std::vector<long long> pre(groups.size(), 0), todo(groups.size(), 0);
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        Group &G = *groups[gi];
        todo[gi] = std::min(units, G.max_units - G.done_units);
        if (todo[gi] <= 0 || !(G.kind == 2 || G.kind == 6) || G.tuned) continue;
        if (G.tune_key.empty()) G.tune_key = tune_key(*this, G);
        if (!getenv("MCSGPU_NO_TUNE_CACHE")) {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            auto it = g_tune_cache.find(G.tune_key);
            if (it != g_tune_cache.end()) {
                G.C = it->second.first;
                G.threads = it->second.second;
                G.tuned = 1;
                continue;
            }
        }
        // every candidate's kernel is loaded before any is timed (CUDA loads a
        // kernel at its first launch, which would count against the first
        // candidate); once per process and device
        {
            static std::mutex m;
            static bool loaded[64];
            std::lock_guard<std::mutex> lock(m);
            if (device >= 0 && device < 64 && !loaded[device]) {
                if (preload_kernels_main() == cudaSuccess) preload_kernels_cluster();
                cudaGetLastError();
                loaded[device] = true;
            }
        }
        long long u = 0;
        const long long probe = std::max<long long>(1, std::min<long long>(4, todo[gi] / (2 * (long long)G.candidates.size() + 1)));
        G.cand_ms.assign(G.candidates.size(), 1e30);
        for (size_t ci = 0; ci < G.candidates.size() && u + probe <= todo[gi]; ++ci) {
            int C = G.candidates[ci].first, th = G.candidates[ci].second;
            CUDA_TRY(cudaEventRecord(ev_a, stream));
            cudaError_t e = launch_group(G, C, th, probe, stream);
            if (e != cudaSuccess) { cudaGetLastError(); continue; }
            CUDA_TRY(cudaEventRecord(ev_b, stream));
            CUDA_TRY(cudaEventSynchronize(ev_b));
            float ms = 0;
            cudaEventElapsedTime(&ms, ev_a, ev_b);
            G.cand_ms[ci] = ms / probe;
            launches++;
            u += probe;
        }
        size_t best = 0;
        for (size_t ci = 1; ci < G.candidates.size(); ++ci) if (G.cand_ms[ci] < G.cand_ms[best]) best = ci;
        if (getenv("MCSGPU_TRACE")) {
            fprintf(stderr, "mcsgpu trace: autotune group %zu (C:threads ms/unit):", gi);
            for (size_t ci = 0; ci < G.candidates.size(); ++ci)
                fprintf(stderr, " %d:%d %.4f", G.candidates[ci].first, G.candidates[ci].second, G.cand_ms[ci]);
            fprintf(stderr, "\n");
        }
        G.C = G.candidates[best].first;
        G.threads = G.candidates[best].second;
        G.tuned = 1;
        pre[gi] = u;
        if (G.cand_ms[best] < 1e29) {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            g_tune_cache[G.tune_key] = {G.C, G.threads};
        }
    }
    rc = run_groups(todo, pre, nullptr);
    if (rc != MCS_OK) return rc;
    for (size_t gi = 0; gi < groups.size(); ++gi)
        if (todo[gi] > 0) groups[gi]->done_units += todo[gi];
    return MCS_OK;
}

// 2. the groups' units: each group on its own stream, side by side on the
// device (MCSGPU_TRACE=1 prints each group's schedule and device time to
// stderr).  ev0 is recorded on `stream` before the call.  With `failed`, a
// group whose launch is refused (a configuration error, which leaves the
// context usable) adds its replicas there and the others go on; an error at
// the synchronisation is returned.
int Batch::run_groups(const std::vector<long long> &todo, const std::vector<long long> &pre, std::vector<int> *failed,
                      std::vector<float> *group_ms)
{
    const bool multi = groups.size() > 1;
    while (multi && gstreams.size() < groups.size()) {
        cudaStream_t gs = nullptr;
        CUDA_TRY(cudaStreamCreateWithFlags(&gs, cudaStreamNonBlocking));
        gstreams.push_back(gs);
        cudaEvent_t ge = nullptr;
        CUDA_TRY(cudaEventCreateWithFlags(&ge, cudaEventDisableTiming));
        gevents.push_back(ge);
    }
    // tiled groups (a large lattice in global memory, whose every sweep is a
    // few short launches over the whole device) run on streams of the
    // device's highest priority, so that their CTAs are placed first and the
    // resident and cluster groups fill the SMs around them: without it a
    // served stream's large lattices crawl behind the other groups' CTAs and
    // finish last (served makespan 1.10-1.16 s against 0.94-1.06 s)
    bool any_tiled = false;
    for (const auto &g : groups) any_tiled |= g->kind == 3;
    while (multi && any_tiled && gstreams_hi.size() < groups.size()) {
        int least = 0, greatest = 0;
        CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        cudaStream_t gs = nullptr;
        CUDA_TRY(cudaStreamCreateWithPriority(&gs, cudaStreamNonBlocking, greatest));
        gstreams_hi.push_back(gs);
    }
    const bool trace = getenv("MCSGPU_TRACE") != nullptr;
    const bool timed = trace || group_ms;
    while (timed && tev.size() < 2 * groups.size()) {  // per-group timing events, kept by the batch
        cudaEvent_t te = nullptr;
        CUDA_TRY(cudaEventCreate(&te));
        tev.push_back(te);
    }
    if (multi) CUDA_TRY(cudaEventRecord(ev_fork, stream));
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        Group &G = *groups[gi];
        const long long n_todo = todo[gi];
        if (n_todo <= 0) continue;
        cudaStream_t gs = multi ? (G.kind == 3 ? gstreams_hi[gi] : gstreams[gi]) : stream;
        if (multi) CUDA_TRY(cudaStreamWaitEvent(gs, ev_fork, 0));
        if (timed) CUDA_TRY(cudaEventRecord(tev[2 * gi], gs));
        cudaError_t e = cudaSuccess;
        const char *what = "";
        if (G.kind == 4 || G.kind == 5) {
            what = "wolff launch: ";
            for (long long u = 0; u < n_todo && e == cudaSuccess; u += G.chunk) {
                long long n = std::min(G.chunk, n_todo - u);
                e = launch_wolff(G.dim, G.geom, d_reps, G.d_ids, (int)G.ids.size(), G.threads, G.smem, n, G.kind == 5, gs);
                if (e == cudaSuccess) launches++;
            }
        } else if (G.kind == 2 || G.kind == 6) {
            what = "resident/cluster launch: ";
            for (long long u = pre[gi]; u < n_todo && e == cudaSuccess; u += G.chunk) {
                long long n = std::min(G.chunk, n_todo - u);
                e = launch_group(G, G.C, G.threads, n, gs);
                if (e == cudaSuccess) launches++;
            }
        } else if (G.kind == 3 && n_todo >= 8) {
            what = "tiled: ";
            if (!G.exec) {
                G.K = (int)std::min<long long>(32, std::max<long long>(1, std::max(n_todo, G.max_units - G.done_units)));
                long long nl = 0;
                CUDA_TRY(cudaStreamBeginCapture(stream2, cudaStreamCaptureModeThreadLocal));
                for (int k = 0; k < G.K && e == cudaSuccess; ++k) e = tiled_unit(G, stream2, &nl);
                cudaGraph_t g0 = nullptr;
                cudaError_t e2 = cudaStreamEndCapture(stream2, &g0);
                if (e == cudaSuccess && e2 == cudaSuccess) {
                    G.graph = g0;
                    e = cudaGraphInstantiate(&G.exec, G.graph, 0);
                    G.per_graph = nl;
                } else {
                    if (g0) cudaGraphDestroy(g0);
                    if (e == cudaSuccess) e = e2;
                    what = "capture: ";
                }
            }
            long long u = 0;
            for (; e == cudaSuccess && u + G.K <= n_todo; u += G.K) {
                e = cudaGraphLaunch(G.exec, gs);
                if (e == cudaSuccess) launches += G.per_graph;
            }
            for (; e == cudaSuccess && u < n_todo; ++u) e = tiled_unit(G, gs, &launches);
        } else {
            what = "tiled: ";
            for (long long u = 0; e == cudaSuccess && u < n_todo; ++u) e = tiled_unit(G, gs, &launches);
        }
        if (e != cudaSuccess) {
            if (!failed) { set_error(std::string(what) + cudaGetErrorString(e)); return MCS_ECUDA; }
            cudaGetLastError();
            failed->insert(failed->end(), G.ids.begin(), G.ids.end());
        }
        if (timed) CUDA_TRY(cudaEventRecord(tev[2 * gi + 1], gs));
        if (multi) {
            CUDA_TRY(cudaEventRecord(gevents[gi], gs));
            CUDA_TRY(cudaStreamWaitEvent(stream, gevents[gi], 0));
        }
    }
    CUDA_TRY(cudaEventRecord(ev1, stream));
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { set_error(std::string("CUDA error in run: ") + cudaGetErrorString(e)); return MCS_ECUDA; }
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    device_ms += ms;
    last_ms = ms;
    if (group_ms) {
        group_ms->assign(groups.size(), -1.f);
        for (size_t gi = 0; gi < groups.size(); ++gi)
            if (todo[gi] > 0) cudaEventElapsedTime(&(*group_ms)[gi], tev[2 * gi], tev[2 * gi + 1]);
        cudaGetLastError();
    }
    if (trace) {
        for (size_t gi = 0; gi < groups.size(); ++gi) {
            const Group &G = *groups[gi];
            float gms = -1.f;
            if (todo[gi] > 0) cudaEventElapsedTime(&gms, tev[2 * gi], tev[2 * gi + 1]);
            long long sites = 0, maxn = 0;
            for (int id : G.ids) { sites += replicas[id]->hm.N; maxn = std::max<long long>(maxn, replicas[id]->hm.N); }
            fprintf(stderr, "mcsgpu trace: group %zu kind %d dim %d C %d threads %d replicas %zu sites %lld max %lld: %.3f ms\n",
                    gi, G.kind, G.dim, G.C, G.threads, G.ids.size(), sites, maxn, gms);
        }
        fprintf(stderr, "mcsgpu trace: step %.3f ms\n", ms);
        cudaGetLastError();
    }
    return MCS_OK;
}

// One server step: every replica of the groups advances by min(quota,
// remaining units).  A small kernel first sets each replica's stop unit
// (u + quota) on the device; the host tracks the same progress.
int Batch::advance_quota(std::vector<int> *failed)
{
    if (groups.empty()) return MCS_OK;
    std::vector<long long> todo(groups.size(), 0), pre(groups.size(), 0);
    std::vector<int> active;
    for (size_t gi = 0; gi < groups.size(); ++gi)
        for (int id : groups[gi]->ids) {
            const Rep &R = replicas[id]->rep;
            const long long n = std::min(R.quota, replicas[id]->hm.units_total - R.u);
            if (n <= 0) continue;
            todo[gi] = std::max(todo[gi], n);
            active.push_back(id);
        }
    if (active.empty()) return MCS_OK;
    if (!d_stop) {
        CUDA_TRY(buf_alloc(device, (void **)&d_stop, (size_t)slot_capacity * sizeof(StopItem)));
        CUDA_TRY(cudaMallocHost(&h_stop, (size_t)slot_capacity * sizeof(StopItem)));
    }
    // one copy of (replica, quota) pairs from page-locked memory and one small
    // kernel set every replica's quota and stop unit for this step
    CUDA_TRY(cudaStreamSynchronize(stream));  // the previous step's copy has been consumed
    for (size_t k = 0; k < active.size(); ++k) {
        h_stop[k].id = active[k];
        h_stop[k].pad = 0;
        h_stop[k].quota = replicas[active[k]]->rep.quota;
    }
    CUDA_TRY(cudaMemcpyAsync(d_stop, h_stop, active.size() * sizeof(StopItem), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaEventRecord(ev0, stream));
    CUDA_TRY(launch_set_stop(d_reps, d_stop, (int)active.size(), stream));
    launches++;
    std::vector<int> fl;
    std::vector<float> gms;
    int rc = run_groups(todo, pre, &fl, &gms);
    if (rc != MCS_OK) return rc;
    std::vector<char> bad(replicas.size(), 0);
    for (int i : fl) bad[i] = 1;
    for (int id : active) {
        if (bad[id]) continue;
        Rep &R = replicas[id]->rep;
        R.u = std::min(replicas[id]->hm.units_total, R.u + R.quota);
    }
    // quotas follow the measured device time: a group whose launches took t ms
    // for its largest quota scales its members' quotas by quota_ms / t (at most
    // x4 or /4 per step), so that every group's share of a step takes about
    // quota_ms whatever its schedule and however the device is shared (the
    // next step's stop kernel carries the new quotas to the device)
    if (quota_ms > 0) {
        for (size_t gi = 0; gi < groups.size(); ++gi) {
            if (todo[gi] <= 0 || gms[gi] <= 0.f) continue;
            const double f = std::min(4.0, std::max(0.25, quota_ms / (double)gms[gi]));
            for (int id : groups[gi]->ids) {
                Rep &R = replicas[id]->rep;
                R.quota = std::max(1LL, std::min((long long)llround((double)R.quota * f), replicas[id]->hm.units_total));
            }
        }
    }
    if (failed) failed->insert(failed->end(), fl.begin(), fl.end());
    return MCS_OK;
}

int Batch::sync_descriptors()
{
    const int nrep = (int)replicas.size();
    if (!prepared || !d_reps || nrep == 0) return MCS_OK;
    std::vector<Rep> host(nrep);
    CUDA_TRY(cudaMemcpy(host.data(), d_reps, nrep * sizeof(Rep), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nrep; ++i) {  // progress travels with the replica
        replicas[i]->rep.u = host[i].u;
        replicas[i]->rep.m = host[i].m;
        replicas[i]->rep.frames_written = host[i].frames_written;
    }
    final_reps.swap(host);
    return MCS_OK;
}

void Batch::release_groups()
{
    groups.clear();
    buf_free(d_reps);
    d_reps = nullptr;
    prepared = false;
}

int Batch::collect()
{
    const int nrep = (int)replicas.size();
    int rc = sync_descriptors();
    if (rc != MCS_OK) return rc;
    std::vector<Replica *> rs;
    for (auto &r : replicas) rs.push_back(r.get());
    rc = fetch_result_blocks(rs, device);
    if (rc != MCS_OK) return rc;
    site_updates = 0;
    for (int i = 0; i < nrep; ++i) {
        long long st[S_NSTAT];
        const Replica &r = *replicas[i];
        memcpy(st, r.rblock.data() + (r.stats_off - r.acc_off), sizeof st);
        site_updates += r.hm.alg == 0 ? st[S_VISITS] : st[S_FLIPPED];
    }
    return MCS_OK;
}

int Batch::run()
{
    device_ms = 0;
    long long maxu = 0;
    for (auto &r : replicas) maxu = std::max(maxu, r->hm.units_total);
    int rc = advance(maxu);
    if (rc != MCS_OK) return rc;
    return collect();
}

int Batch::result(int i, mcs_result *res)
{
    if (i < 0 || i >= (int)replicas.size()) { set_error("replica index out of range"); return MCS_EINVAL; }
    if ((int)final_reps.size() != (int)replicas.size()) { set_error("batch has not been run"); return MCS_EINVAL; }
    int rc = replica_results(replicas[i].get(), final_reps[i], res);
    if (rc == MCS_OK && res) res->device_ms = device_ms;
    return rc;
}

}  // namespace mcs

// ====================================================================== C ABI
using namespace mcs;

extern "C" {

const char *mcs_last_error(void) { return get_error().c_str(); }
int mcs_abi_version(void) { return 1; }

// Host-compile check, exported for the CPU tests and deliberately not declared
// in include/mcsgpu.h: compiles `problem` on the host (no device call) and
// returns an FNV-1a digest of its arena image and descriptor, the bytes a
// batch uploads.  With `template_problem` set, that problem is compiled first
// and `problem` is compiled from its template (*reused tells whether the
// template's structure was taken), so a test can check that the template path
// and a full compile give the same bytes.
// Host-compile facts, exported for the CPU tests and not declared in
// include/mcsgpu.h: info[0..7] = geometry (0 general, 1 square), cluster
// schedule applies, regular square measurement, sites, Lx, Ly, colours,
// every correlated pair (v, v).
int mcs_test_compile_info(const mcs_problem *problem, const mcs_options *options, int32_t *info)
{
    try {
        mcs_options def;
        memset(&def, 0, sizeof def);
        Replica r;
        int rc = build_replica(problem, options ? options : &def, &r, false);
        if (rc != MCS_OK) return rc;
        const HostModel &m = r.hm;
        const int32_t v[8] = {m.geom, m.cluster_ok, m.meas_regular, m.N, m.Lx, m.Ly, m.ncol, m.pair_identity};
        for (int k = 0; k < 8; ++k) info[k] = v[k];
        return MCS_OK;
    } catch (const std::exception &e) {
        set_error(e.what());
        return MCS_EINVAL;
    }
}

int mcs_test_compile_digest(const mcs_problem *template_problem, const mcs_problem *problem,
                            const mcs_options *options, uint64_t *digest, int32_t *reused)
{
    try {
        mcs_options def;
        memset(&def, 0, sizeof def);
        const mcs_options *o = options ? options : &def;
        std::shared_ptr<const ModelTemplate> t;
        if (template_problem) {
            Replica a;
            int rc = build_replica(template_problem, o, &a, false);
            if (rc != MCS_OK) return rc;
            if (template_problem->model != MCS_ISING) t = make_template(template_problem, a.hm);
        }
        Replica r;
        bool re = false;
        int rc = build_replica(problem, o, &r, false, t.get(), &re);
        if (rc != MCS_OK) return rc;
        uint64_t h = 1469598103934665603ULL;
        auto mix = [&h](const void *d, size_t n) {
            const unsigned char *c = (const unsigned char *)d;
            for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ULL; }
        };
        mix(r.staging.data(), r.staging.size());
        mix(&r.rep, sizeof(Rep));
        if (digest) *digest = h;
        if (reused) *reused = re ? 1 : 0;
        return MCS_OK;
    } catch (const std::exception &e) {
        set_error(e.what());
        return MCS_EINVAL;
    }
}
const char *mcs_build_info(void)
{
    return "mcsgpu: sm_103a Monte Carlo spin-lattice engine (Ising/XY/Heisenberg; Metropolis colour sweeps, "
           "Philox4x32-10, FP32 updates with FP64 accumulation)";
}

int mcs_solve(const mcs_problem *problem, const mcs_options *options, mcs_result *result)
{
    try {
        mcs_options def;
        memset(&def, 0, sizeof def);
        if (!options) options = &def;
        Batch b;
        int rc = b.init(options->device);
        if (rc != MCS_OK) return rc;
        int idx = 0;
        rc = b.add(problem, options, &idx);
        if (rc != MCS_OK) return rc;
        rc = b.run();
        if (rc != MCS_OK) return rc;
        return b.result(idx, result);
    } catch (const std::exception &e) {
        set_error(std::string("exception: ") + e.what());
        return MCS_ECUDA;
    }
}

struct mcs_batch {
    mcs::Batch b;
};

int mcs_batch_create(int32_t device, mcs_batch **out)
{
    if (!out) return MCS_EINVAL;
    mcs_batch *x = new mcs_batch();
    int rc = x->b.init(device);
    if (rc != MCS_OK) { delete x; return rc; }
    *out = x;
    return MCS_OK;
}
int mcs_batch_add(mcs_batch *b, const mcs_problem *problem, const mcs_options *options, int32_t *replica)
{
    if (!b) return MCS_EINVAL;
    mcs_options def;
    memset(&def, 0, sizeof def);
    int idx = 0;
    int rc = b->b.add(problem, options ? options : &def, &idx);
    if (replica) *replica = idx;
    return rc;
}
int mcs_batch_run(mcs_batch *b) { return b ? b->b.run() : MCS_EINVAL; }
int mcs_batch_prepare(mcs_batch *b) { return b ? b->b.prepare() : MCS_EINVAL; }
int mcs_batch_advance(mcs_batch *b, int64_t units, double *device_ms)
{
    if (!b) return MCS_EINVAL;
    int rc = b->b.advance(units);
    if (rc == MCS_OK) rc = b->b.collect();
    if (device_ms) *device_ms = b->b.last_ms;
    return rc;
}
int mcs_batch_result(mcs_batch *b, int32_t replica, mcs_result *result) { return b ? b->b.result(replica, result) : MCS_EINVAL; }
int mcs_batch_stats(mcs_batch *b, double *device_ms, int64_t *site_updates, int32_t *launches)
{
    if (!b) return MCS_EINVAL;
    if (device_ms) *device_ms = b->b.device_ms;
    if (site_updates) *site_updates = b->b.site_updates;
    if (launches) *launches = (int32_t)b->b.launches;
    return MCS_OK;
}
int mcs_batch_schedule(mcs_batch *b, int32_t group, int32_t *kind, int32_t *cluster, int32_t *threads,
                       int32_t *replicas)
{
    if (!b) return MCS_EINVAL;
    if (group < 0 || group >= (int32_t)b->b.groups.size()) { set_error("group index out of range"); return MCS_EINVAL; }
    const Group &G = *b->b.groups[group];
    if (kind) *kind = G.kind;
    if (cluster) *cluster = G.C;
    if (threads) *threads = G.threads;
    if (replicas) *replicas = (int32_t)G.ids.size();
    return MCS_OK;
}
int mcs_batch_memory(mcs_batch *b, uint64_t *device_bytes, uint64_t *readback_bytes)
{
    if (!b) return MCS_EINVAL;
    uint64_t dev = 0, rb = 0;
    for (auto &sl : b->b.shared_lists) dev += sl.second->bytes;
    for (auto &r : b->b.replicas) {
        dev += r->bytes + sizeof(Rep);
        rb += sizeof(Rep) + r->nacc * sizeof(double) + (C_NINT + S_NSTAT) * sizeof(long long);
    }
    if (device_bytes) *device_bytes = dev;
    if (readback_bytes) *readback_bytes = rb;
    return MCS_OK;
}
void mcs_batch_destroy(mcs_batch *b) { delete b; }

}  // extern "C"

// ====================================================================== parallel tempering
struct mcs_pt {
    mcs::Batch b;
    int nt = 0;
    std::vector<double> betas;
    int *d_perm = nullptr;
    long long *d_acc = nullptr, *d_att = nullptr;
    unsigned long long seed = 0;
    double ms = 0;
    bool ran = false;
    ~mcs_pt()
    {
        if (d_perm) cudaFree(d_perm);
        if (d_acc) cudaFree(d_acc);
        if (d_att) cudaFree(d_att);
    }
};

extern "C" int mcs_pt_create(const mcs_problem *problem, const mcs_options *options, const double *betas,
                             int32_t n_temps, mcs_pt **out)
{
    if (!problem || !betas || !out || n_temps < 2) { set_error("parallel tempering needs a problem and >= 2 temperatures"); return MCS_EINVAL; }
    if (problem->model == MCS_ISING) { set_error("parallel tempering is built for the XY and Heisenberg models"); return MCS_EUNSUPPORTED; }
    if (problem->algorithm != MCS_METROPOLIS) { set_error("parallel tempering runs Metropolis sweeps"); return MCS_EUNSUPPORTED; }
    for (int k = 0; k < n_temps; ++k)
        if (!(betas[k] > 0)) { set_error("betas must be positive"); return MCS_EINVAL; }
    mcs_options def;
    memset(&def, 0, sizeof def);
    if (!options) options = &def;
    std::unique_ptr<mcs_pt> pt(new mcs_pt());
    int rc = pt->b.init(options->device);
    pt->b.balance = 0;  // the exchange kernel needs every temperature in one kernel group
    if (rc != MCS_OK) return rc;
    pt->nt = n_temps;
    pt->seed = options->seed;
    for (int k = 0; k < n_temps; ++k) {
        mcs_options o = *options;
        o.seed = options->seed + 0x9E3779B97F4A7C15ULL * (unsigned long long)(k + 1);
        if (o.schedule == 0) o.schedule = 2;
        int idx = 0;
        rc = pt->b.add(problem, &o, &idx);
        if (rc != MCS_OK) return rc;
        pt->b.replicas[idx]->rep.beta = (float)betas[k];
        pt->betas.push_back(betas[k]);
    }
    if (pt->b.replicas[0]->hm.upm != 1) { set_error("parallel tempering measures after every sweep (ninterval = N)"); return MCS_EINVAL; }
    *out = pt.release();
    return MCS_OK;
}

extern "C" int mcs_pt_run(mcs_pt *pt)
{
    if (!pt) return MCS_EINVAL;
    Batch &b = pt->b;
    int rc = b.prepare();
    if (rc != MCS_OK) return rc;
    if (b.groups.size() != 1) { set_error("parallel tempering replicas must form one kernel group"); return MCS_EINVAL; }
    Group &G = *b.groups[0];
    // the group's first configuration (the only one when MCSGPU_COPIES or
    // MCSGPU_FORCE leave one); with several, the probe below picks
    int C = 0, threads = G.threads;
    if (!G.candidates.empty()) { C = G.candidates[0].first; threads = G.candidates[0].second; }
    const int nt = pt->nt;
    CUDA_TRY(cudaMalloc(&pt->d_perm, nt * sizeof(int)));
    CUDA_TRY(cudaMalloc(&pt->d_acc, nt * sizeof(long long)));
    CUDA_TRY(cudaMalloc(&pt->d_att, nt * sizeof(long long)));
    std::vector<int> perm(nt);
    for (int k = 0; k < nt; ++k) perm[k] = k;
    CUDA_TRY(cudaMemcpy(pt->d_perm, perm.data(), nt * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(pt->d_acc, 0, nt * sizeof(long long)));
    CUDA_TRY(cudaMemset(pt->d_att, 0, nt * sizeof(long long)));
    const long long total = G.max_units;
    auto sweep = [&](cudaStream_t s) -> cudaError_t {
        cudaError_t e = b.launch_group(G, C, threads, 1, s);
        if (e != cudaSuccess) return e;
        return launch_pt_exchange(b.d_reps, nt, pt->d_perm, pt->seed ^ 0x5054ULL, pt->d_acc, pt->d_att, s);
    };
    CUDA_TRY(cudaEventRecord(b.ev0, b.stream));
    long long u = 0;
    // configuration: time each candidate of the group (one CTA per replica, or
    // copies of each replica over a cluster) on real sweeps + exchanges
    if (G.kind == 2 && G.candidates.size() > 1 && total >= 16 * (long long)G.candidates.size()) {
        float best = 1e30f;
        for (auto &cand : G.candidates) {
            const int cC = cand.first, cth = cand.second;
            CUDA_TRY(cudaEventRecord(b.ev_a, b.stream));
            cudaError_t e = cudaSuccess;
            for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
                e = b.launch_group(G, cC, cth, 1, b.stream);
                if (e == cudaSuccess)
                    e = launch_pt_exchange(b.d_reps, nt, pt->d_perm, pt->seed ^ 0x5054ULL, pt->d_acc, pt->d_att, b.stream);
            }
            if (e != cudaSuccess) { set_error(std::string("parallel tempering probe: ") + cudaGetErrorString(e)); return MCS_ECUDA; }
            CUDA_TRY(cudaEventRecord(b.ev_b, b.stream));
            CUDA_TRY(cudaEventSynchronize(b.ev_b));
            float ms = 0;
            cudaEventElapsedTime(&ms, b.ev_a, b.ev_b);
            if (ms < best) { best = ms; C = cC; threads = cth; }
            if (getenv("MCSGPU_TRACE"))
                fprintf(stderr, "mcsgpu trace: parallel tempering candidate %d:%d %.4f ms per sweep + exchange\n", cC, cth,
                        ms / 4);
            u += 4;
        }
    }
    const int K = 32;
    if (total - u >= 2 * K) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(b.stream2, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < K && e == cudaSuccess; ++k) e = sweep(b.stream2);
        cudaError_t e2 = cudaStreamEndCapture(b.stream2, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            set_error(std::string("parallel tempering capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
            return MCS_ECUDA;
        }
        CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
        for (; u + K <= total; u += K) CUDA_TRY(cudaGraphLaunch(exec, b.stream));
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
    }
    for (; u < total; ++u) CUDA_TRY(sweep(b.stream));
    CUDA_TRY(cudaEventRecord(b.ev1, b.stream));
    CUDA_TRY(cudaStreamSynchronize(b.stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, b.ev0, b.ev1);
    pt->ms = ms;
    b.device_ms = ms;
    G.done_units = total;
    rc = b.collect();
    pt->ran = rc == MCS_OK;
    return rc;
}

extern "C" int mcs_pt_result(mcs_pt *pt, int32_t k, mcs_result *result)
{
    if (!pt || !pt->ran) { set_error("parallel tempering has not been run"); return MCS_EINVAL; }
    if (k < 0 || k >= pt->nt) { set_error("temperature index out of range"); return MCS_EINVAL; }
    // the accumulators of temperature k live in the arena allocated for replica k
    return pt->b.result(k, result);
}

extern "C" int mcs_pt_stats(mcs_pt *pt, double *swap_acceptance, double *device_ms, int64_t *site_updates)
{
    if (!pt || !pt->ran) { set_error("parallel tempering has not been run"); return MCS_EINVAL; }
    std::vector<long long> a(pt->nt), t(pt->nt);
    CUDA_TRY(cudaMemcpy(a.data(), pt->d_acc, pt->nt * sizeof(long long), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(t.data(), pt->d_att, pt->nt * sizeof(long long), cudaMemcpyDeviceToHost));
    if (swap_acceptance)
        for (int k = 0; k + 1 < pt->nt; ++k) swap_acceptance[k] = t[k] ? (double)a[k] / (double)t[k] : 0.0;
    if (device_ms) *device_ms = pt->ms;
    if (site_updates) *site_updates = pt->b.site_updates;
    return MCS_OK;
}

extern "C" void mcs_pt_destroy(mcs_pt *pt) { delete pt; }
