// mcs_model.cpp -- model compiler.
//
// Input: the flattened arrays of one MCMainFunction call (isingLib.c:277-335,
// heisenbergLib.c:504-583).  Output: the engine's device layout
//   * greedy colouring of the bond graph in site order; sites renumbered into
//     colour-major "sweep index" order (contiguous colour ranges);
//   * 2D square lattices detected and given an arithmetic neighbour rule;
//     everything else keeps an ELL neighbour table [link][site];
//   * O(n): exchange matrices de-duplicated into a small class table, the
//     anisotropy vectors into a D table;
//   * Ising: directed couplings K*|s_i|*|s_j| grouped into <= 4 classes and
//     sites into <= 4 types; per type an exact acceptance table indexed by the
//     neighbour-sign pattern (thresholds ceil(exp(corr)*2^32)).
#include "mcs_model.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <map>
#include <set>
#include <string>
#include <unordered_map>
#include <utility>

namespace mcs {

// De-duplication of K-double keys (bitwise equality).  Most lattices repeat a
// handful of values in long runs, so the previous hit and a short linear scan
// answer almost every lookup; a hash map covers the rest.
template <int K>
struct ClassTable {
    std::vector<std::array<double, K>> keys;
    std::unordered_map<std::string, int> map;
    int last = -1;
    int find_or_add(const double *v)
    {
        if (last >= 0 && memcmp(keys[last].data(), v, sizeof(double) * K) == 0) return last;
        if (keys.size() <= 16) {
            for (size_t c = 0; c < keys.size(); ++c)
                if (memcmp(keys[c].data(), v, sizeof(double) * K) == 0) return last = (int)c;
        } else {
            auto it = map.find(std::string((const char *)v, sizeof(double) * K));
            if (it != map.end()) return last = it->second;
        }
        std::array<double, K> a;
        memcpy(a.data(), v, sizeof(double) * K);
        keys.push_back(a);
        int c = (int)keys.size() - 1;
        if (keys.size() == 17)
            for (size_t q = 0; q < keys.size(); ++q)
                map[std::string((const char *)keys[q].data(), sizeof(double) * K)] = (int)q;
        else if (keys.size() > 17)
            map[std::string((const char *)v, sizeof(double) * K)] = c;
        return last = c;
    }
};

void philox_host(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, unsigned long long seed, uint32_t out[4])
{
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double u24d(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }
static const double kTwoPi = 6.28318530717958647692528676655900577;

static void eng_dir(int dim, uint32_t w0, uint32_t w1, double d[3])
{
    if (dim == 2) {
        double phi = kTwoPi * u24d(w0);
        d[0] = cos(phi); d[1] = sin(phi); d[2] = 0;
    } else {
        double zz = 2.0 * u24d(w0) - 1.0;
        double phi = kTwoPi * u24d(w1);
        double rho = sqrt(fmax(0.0, 1.0 - zz * zz));
        d[0] = rho * cos(phi); d[1] = rho * sin(phi); d[2] = zz;
    }
}

#define FAIL(code, msg)           \
    do {                          \
        if (err) *err = (msg);    \
        return (code);            \
    } while (0)

// Bitwise equality of two 9-double coupling matrices (inline: this runs once
// per link).
static inline bool same_bits9(const double *a, const double *b)
{
    uint64_t d = 0;
    for (int k = 0; k < 9; ++k) {
        uint64_t x, y;
        memcpy(&x, a + k, 8);
        memcpy(&y, b + k, 8);
        d |= x ^ y;
    }
    return d == 0;
}

// The structural inputs of p equal those recorded in the template, bit for bit.
static bool same_structure(const StructInputs &in, const mcs_problem *p)
{
    if (in.model != p->model || in.alg != p->algorithm || in.N != p->n_sites || in.z != p->max_links) return false;
    if (in.n_circuits != p->n_circuits || in.n_lat != p->n_lat || in.n_group != p->n_group ||
        in.max_group != p->max_group || in.n_rorb != p->n_rorb || in.n_in_cluster != p->n_in_cluster ||
        in.ignore_offdiag != p->ignore_offdiag || in.has_rlink != (p->r_link != nullptr))
        return false;
    auto eq = [](const auto &v, const void *q) {
        return v.empty() || (q && memcmp(v.data(), q, v.size() * sizeof(v[0])) == 0);
    };
    return eq(in.nlink, p->nlink) && eq(in.linked_orb, p->linked_orb) && eq(in.circuits, p->circuits) &&
           eq(in.corr_pair, p->corr_pair) && eq(in.group_list, p->group_list) && eq(in.r_orb, p->r_orb) &&
           eq(in.r_cluster, p->r_cluster) && eq(in.r_link, p->r_link) && eq(in.init_spin, p->init_spin);
}

std::shared_ptr<const ModelTemplate> make_template(const mcs_problem *p, const HostModel &m)
{
    auto t = std::make_shared<ModelTemplate>();
    t->hm = m;
    t->linkcls = std::move(t->hm.linkcls);
    std::vector<int>().swap(t->hm.linkcls);
    std::vector<float>().swap(t->hm.init_vec);
    std::vector<int8_t>().swap(t->hm.init_sigma);
    StructInputs &in = t->in;
    in.model = p->model; in.alg = p->algorithm; in.N = p->n_sites; in.z = p->max_links;
    in.n_circuits = p->n_circuits; in.n_lat = p->n_lat; in.n_group = p->n_group; in.max_group = p->max_group;
    in.n_rorb = p->n_rorb; in.n_in_cluster = p->n_in_cluster; in.ignore_offdiag = p->ignore_offdiag;
    in.has_rlink = p->r_link != nullptr;
    const size_t N = p->n_sites, z = p->max_links;
    auto cp = [](auto &v, const auto *q, size_t n) { if (q && n) v.assign(q, q + n); };
    cp(in.nlink, p->nlink, N);
    cp(in.linked_orb, p->linked_orb, N * z);
    cp(in.circuits, p->circuits, 3 * (size_t)p->n_circuits);
    cp(in.corr_pair, p->corr_pair, 2 * (size_t)p->n_lat);
    cp(in.group_list, p->group_list, (size_t)p->n_group * p->max_group);
    cp(in.r_orb, p->r_orb, (size_t)p->n_rorb);
    cp(in.r_cluster, p->r_cluster, (size_t)p->n_rorb * p->n_in_cluster);
    cp(in.r_link, p->r_link, (size_t)p->n_rorb * z);
    cp(in.init_spin, p->init_spin, N);
    return t;
}

// O(n) site classes (anisotropy vector and spin length) in the sweep order
// `sites`: stype per sweep index, the class table dtab [ndc][4], has_d.
static int onsite_classes(const mcs_problem *p, int dim, int N, const std::vector<int> &sites,
                          std::vector<uint8_t> *stype, std::vector<float> *dtab, int *ndc, int *has_d, std::string *err)
{
    ClassTable<4> dcls;
    stype->assign(N, 0);
    bool anyd = false;
    for (int k = 0; k < N; ++k) {
        int i = sites[k];
        double v[4] = {p->init_d[3 * (size_t)i], p->init_d[3 * (size_t)i + 1], p->init_d[3 * (size_t)i + 2],
                       fabs(p->init_spin[i])};
        if (dim == 2) v[2] = 0.0;
        anyd |= v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0;
        int c = dcls.find_or_add(v);
        if (c > 255) FAIL(MCS_EUNSUPPORTED, "more than 256 distinct (anisotropy, spin length) site classes");
        (*stype)[k] = (uint8_t)c;
    }
    *ndc = (int)dcls.keys.size();
    *has_d = anyd ? 1 : 0;
    dtab->resize(4 * dcls.keys.size());
    for (size_t c = 0; c < dcls.keys.size(); ++c)
        for (int k = 0; k < 4; ++k) (*dtab)[4 * c + k] = (float)dcls.keys[c][k];
    return MCS_OK;
}

static int compile_program_state(const mcs_problem *p, const mcs_options *o, HostModel *m, int dim, std::string *err);

int compile_model(const mcs_problem *p, const mcs_options *o, HostModel *m, std::string *err,
                  const ModelTemplate *tmpl, bool *reused)
{
    if (reused) *reused = false;
    if (!p) FAIL(MCS_EINVAL, "null problem");
    if (p->model < 1 || p->model > 3) FAIL(MCS_EINVAL, "model must be 1 (Ising), 2 (XY) or 3 (Heisenberg)");
    if (p->algorithm != 0 && p->algorithm != 1) FAIL(MCS_EINVAL, "algorithm must be 0 (Metropolis) or 1 (Wolff)");
    const int N = p->n_sites, z = p->max_links;
    if (N <= 0) FAIL(MCS_EINVAL, "empty lattice (no sites)");
    if (N > (1 << 28)) FAIL(MCS_EINVAL, "lattice too large");
    if (z < 0 || z > MCS_MAXZ) FAIL(MCS_EINVAL, "maxNLinking out of range (0..32)");
    if (!p->init_spin || !p->nlink || (z > 0 && (!p->link_strength || !p->linked_orb)))
        FAIL(MCS_EINVAL, "missing site or link arrays");
    if (p->nthermal < 0 || p->nsweep < 1) FAIL(MCS_EINVAL, "nsweep must be >= 1 and nthermal >= 0");
    if (p->ninterval < 1) FAIL(MCS_EINVAL, "ninterval must be >= 1");
    if (p->n_lat < 1 || !p->corr_pair) FAIL(MCS_EINVAL, "corrOrbPair must hold at least one pair");
    if (p->n_rorb < 1 || !p->r_orb || p->n_in_cluster < 1 || !p->r_cluster)
        FAIL(MCS_EINVAL, "renormalisation lists (rOrb, rOrbCluster) must be non-empty");
    if (p->model != 1 && p->n_group > MCS_MAXG) FAIL(MCS_EUNSUPPORTED, "more than 8 orbital groups");
    if (p->n_group < 0 || (p->n_group > 0 && (p->max_group < 1 || !p->group_list)))
        FAIL(MCS_EINVAL, "bad orbital-group list");
    if (p->n_circuits < 0 || (p->n_circuits > 0 && !p->circuits)) FAIL(MCS_EINVAL, "bad circuit list");
    if (p->spin_frames < 0 || p->spin_frames > p->nsweep)
        FAIL(MCS_EINVAL, "spinFrame must be in [0, nsweep]");
    if (o && o->fp64_update)
        FAIL(MCS_EUNSUPPORTED, "fp64_update: the engine updates spins in FP32 only; the FP64 reference of the same "
                               "stream is the oracle's engine-stream mode");
    const int dim = p->model == 1 ? 1 : (p->model == 2 ? 2 : 3);
    if (dim > 1 && !p->init_d) FAIL(MCS_EINVAL, "initD missing");
    m->model = p->model; m->dim = dim; m->alg = p->algorithm; m->N = N; m->zmax = z;
    m->h = p->h; m->flunc = p->flunc;
    m->seed = o ? o->seed : 0;

    // a problem whose structural inputs equal a validated template's needs no
    // second index validation
    const ModelTemplate *like = (tmpl && dim > 1 && same_structure(tmpl->in, p)) ? tmpl : nullptr;
    if (!like) {
        for (int i = 0; i < N; ++i) {
            if (p->nlink[i] < 0 || p->nlink[i] > z) FAIL(MCS_EINVAL, "nlink out of range");
            for (int l = 0; l < p->nlink[i]; ++l) {
                int j = p->linked_orb[(size_t)i * z + l];
                if (j < 0 || j >= N) FAIL(MCS_EINVAL, "linkedOrb index out of range");
            }
        }
        for (int k = 0; k < 2 * p->n_lat; ++k)
            if (p->corr_pair[k] < 0 || p->corr_pair[k] >= N) FAIL(MCS_EINVAL, "corrOrbPair index out of range");
        for (int k = 0; k < p->n_rorb; ++k)
            if (p->r_orb[k] < 0 || p->r_orb[k] >= N) FAIL(MCS_EINVAL, "rOrb index out of range");
        for (long long k = 0; k < (long long)p->n_rorb * p->n_in_cluster; ++k)
            if (p->r_cluster[k] < 0 || p->r_cluster[k] >= N) FAIL(MCS_EINVAL, "rOrbCluster index out of range");
        if (z > 0 && p->r_link)
            for (long long k = 0; k < (long long)p->n_rorb * z; ++k)
                if (p->r_link[k] < -1 || p->r_link[k] >= N) FAIL(MCS_EINVAL, "linkedOrb_rnorm index out of range");
        for (int k = 0; k < 3 * p->n_circuits; ++k)
            if (p->circuits[k] < 0 || p->circuits[k] >= N) FAIL(MCS_EINVAL, "circuit index out of range");
        for (long long k = 0; k < (long long)p->n_group * p->max_group; ++k)
            if (p->group_list[k] >= N) FAIL(MCS_EINVAL, "orbital-group index out of range");
    }

    // ---------------------------------------------------------------- coupling classes
    // O(n): exchange-matrix classes over all links (exact equality).
    std::vector<int> linkcls((size_t)N * std::max(z, 1), 0);
    if (dim > 1) {
        const bool ign = p->ignore_offdiag > 0;
        ClassTable<9> cls;
        bool anyoff = false;
        // A link whose matrix has the bits of the last matrix seen in the same
        // link slot (translation-invariant lattices repeat the slot pattern
        // site after site), or of the previous link, takes that link's class
        // without a table lookup.
        const double *slotJ[MCS_MAXZ] = {};
        int slotc[MCS_MAXZ] = {};
        const double *prevJ = nullptr;
        int prevc = 0;
        for (int i = 0; i < N; ++i) {
            const int nl = p->nlink[i];
            const double *Ji = p->link_strength + (size_t)i * z * 9;
            // a site with as many links as the previous one and the same bits
            // in every one of them: each link matches the same slot of the
            // previous site, so the slot rule below gives it that slot's class
            // (one block compare instead of one per link)
            if (i > 0 && nl > 0 && nl == p->nlink[i - 1] &&
                memcmp(Ji, Ji - (size_t)z * 9, sizeof(double) * 9 * (size_t)nl) == 0) {
                for (int l = 0; l < nl; ++l) {
                    linkcls[(size_t)i * z + l] = slotc[l];
                    slotJ[l] = Ji + 9 * l;
                }
                prevJ = Ji + 9 * (nl - 1);
                prevc = slotc[nl - 1];
                continue;
            }
            for (int l = 0; l < nl; ++l) {
                const double *J = p->link_strength + ((size_t)i * z + l) * 9;
                int c;
                if (slotJ[l] && same_bits9(J, slotJ[l])) {
                    c = slotc[l];
                } else if (prevJ && same_bits9(J, prevJ)) {
                    c = prevc;
                } else {
                    double v[9];
                    memcpy(v, J, sizeof v);
                    if (ign) v[3] = v[4] = v[5] = v[6] = v[7] = v[8] = 0.0;
                    if (dim == 2) v[2] = v[4] = v[5] = v[7] = v[8] = 0.0;  // XY reads xx,yy,xy,yx (xyLib.c:150-153)
                    for (int k = 3; k < 9; ++k) anyoff |= v[k] != 0.0;
                    c = cls.find_or_add(v);
                }
                linkcls[(size_t)i * z + l] = c;
                slotJ[l] = J; slotc[l] = c;
                prevJ = J; prevc = c;
            }
        }
        if (cls.keys.size() > 65535) FAIL(MCS_EUNSUPPORTED, "too many distinct exchange matrices");
        std::vector<std::vector<double>> tab;
        for (auto &k : cls.keys) tab.push_back(std::vector<double>(k.begin(), k.end()));
        if (tab.empty()) tab.push_back(std::vector<double>(9, 0.0));
        m->njc = (int)tab.size();
        m->fullJ = anyoff ? 1 : 0;
        m->jtab.resize(9 * tab.size());
        m->jtab64.resize(9 * tab.size());
        for (size_t c = 0; c < tab.size(); ++c)
            for (int k = 0; k < 9; ++k) { m->jtab[9 * c + k] = (float)tab[c][k]; m->jtab64[9 * c + k] = tab[c][k]; }
    } else {
        // Ising: classes of Q = K |s_i| |s_j|, site types (|s_i|, class counts)
        ClassTable<1> qcls;
        for (int i = 0; i < N; ++i)
            for (int l = 0; l < p->nlink[i]; ++l) {
                int j = p->linked_orb[(size_t)i * z + l];
                double q = p->link_strength[(size_t)i * z + l] * fabs(p->init_spin[i]) * fabs(p->init_spin[j]);
                linkcls[(size_t)i * z + l] = qcls.find_or_add(&q);
                if (qcls.keys.size() > MCS_MAXC) break;
            }
        std::vector<double> qv;
        for (auto &k : qcls.keys) qv.push_back(k[0]);
        if (qv.size() > MCS_MAXC) FAIL(MCS_EUNSUPPORTED, "Ising model with more than 4 distinct coupling values");
        if (qv.empty()) qv.push_back(0.0);
        m->nclass = (int)qv.size();
        for (int c = 0; c < m->nclass; ++c) m->Q[c] = qv[c];
    }

    // ---------------------------------------------------------------- template
    // same lattice as the template, with the same partition of the links into
    // coupling classes and of the sites into anisotropy classes: the geometry,
    // colouring and measurement lists are the template's; the class values,
    // the program and the initial state are this problem's
    if (like && linkcls == like->linkcls) {
        std::vector<uint8_t> st;
        std::vector<float> dtab;
        int ndc = 0, has_d = 0;
        int rc = onsite_classes(p, dim, N, like->hm.sites, &st, &dtab, &ndc, &has_d, err);
        if (rc != MCS_OK) return rc;
        if (st == like->hm.stype) {
            std::vector<float> jt = std::move(m->jtab);
            std::vector<double> jt64 = std::move(m->jtab64);
            const int njc = m->njc, fullJ = m->fullJ;
            const double h = m->h, flunc = m->flunc;
            const unsigned long long seed = m->seed;
            *m = like->hm;
            m->jtab = std::move(jt); m->jtab64 = std::move(jt64); m->njc = njc; m->fullJ = fullJ;
            m->dtab = std::move(dtab); m->ndc = ndc; m->has_d = has_d;
            m->h = h; m->flunc = flunc; m->seed = seed;
            if (reused) *reused = true;
            return compile_program_state(p, o, m, dim, err);
        }
    }

    // ---------------------------------------------------------------- geometry
    // square lattice: site id = x*Ly + y, four links to (x+-1,y), (x,y+-1),
    // each direction one coupling class; both sides even
    m->geom = MCS_GEOM_ELL;
    if (z >= 4) {
        for (int Ly = 4; Ly <= N / 4 && m->geom == MCS_GEOM_ELL; Ly += 2) {
            if (N % Ly) continue;
            int Lx = N / Ly;
            if (Lx < 4 || (Lx & 1)) continue;
            bool okg = true;
            int code0[4] = {-1, -1, -1, -1};
            // site i = x*Ly + y, with (x, y) stepped along i
            for (int i = 0, x = 0, y = 0; i < N && okg; ++i, y = (y + 1 == Ly) ? (++x, 0) : y + 1) {
                if (p->nlink[i] != 4) { okg = false; break; }
                const int xp = x + 1 == Lx ? 0 : x + 1, xm = x == 0 ? Lx - 1 : x - 1;
                const int yp = y + 1 == Ly ? 0 : y + 1, ym = y == 0 ? Ly - 1 : y - 1;
                int want[4] = {xp * Ly + y, xm * Ly + y, x * Ly + yp, x * Ly + ym};
                int seen = 0;
                for (int l = 0; l < 4; ++l) {
                    int j = p->linked_orb[(size_t)i * z + l];
                    int d = -1;
                    for (int q = 0; q < 4; ++q)
                        if (j == want[q] && !(seen & (1 << q))) { d = q; break; }
                    if (d < 0) { okg = false; break; }
                    seen |= 1 << d;
                    int cc = linkcls[(size_t)i * z + l];
                    if (code0[d] < 0) code0[d] = cc;
                    else if (code0[d] != cc) { okg = false; break; }
                }
            }
            if (okg) {
                m->geom = MCS_GEOM_SQUARE;
                m->Lx = Lx; m->Ly = Ly;
                for (int d = 0; d < 4; ++d) {
                    m->sq_cls[d] = code0[d];
                    if (dim > 1) m->sq_code[d] = code0[d];
                }
            }
        }
    }
    // ---------------------------------------------------------------- colouring
    // A square lattice with even sides gets the parity colouring (x + y) & 1,
    // which is what the greedy colouring in site order produces on it: every
    // earlier neighbour of a site has the other parity.  Other lattices are
    // coloured greedily.
    std::vector<int> colour(N, 0);
    int ncol = 0;
    if (m->geom == MCS_GEOM_SQUARE) {
        for (int x = 0, i = 0; x < m->Lx; ++x)
            for (int y = 0; y < m->Ly; ++y, ++i) colour[i] = (x + y) & 1;
        ncol = 2;
    } else {
    std::vector<int> off(N + 1, 0), adj;
    {
        std::vector<int> degc(N, 0);
        for (int i = 0; i < N; ++i)
            for (int l = 0; l < p->nlink[i]; ++l) {
                int j = p->linked_orb[(size_t)i * z + l];
                if (j == i) continue;
                degc[i]++; degc[j]++;
            }
        for (int i = 0; i < N; ++i) off[i + 1] = off[i] + degc[i];
        adj.resize(off[N]);
        std::vector<int> fill(N, 0);
        for (int i = 0; i < N; ++i)
            for (int l = 0; l < p->nlink[i]; ++l) {
                int j = p->linked_orb[(size_t)i * z + l];
                if (j == i) continue;
                adj[off[i] + fill[i]++] = j;
                adj[off[j] + fill[j]++] = i;
            }
    }
    {
        std::vector<char> used;
        for (int i = 0; i < N; ++i) {
            used.assign(off[i + 1] - off[i] + 2, 0);
            for (int k = off[i]; k < off[i + 1]; ++k) {
                int j = adj[k];
                if (j < i && colour[j] < (int)used.size()) used[colour[j]] = 1;
            }
            int c = 0;
            while (used[c]) ++c;
            colour[i] = c;
            ncol = std::max(ncol, c + 1);
        }
    }
    }
    if (ncol > 64) FAIL(MCS_EUNSUPPORTED, "bond graph needs more than 64 colours");
    m->ncol = ncol;
    m->col_start.assign(ncol + 1, 0);
    for (int i = 0; i < N; ++i) m->col_start[colour[i] + 1]++;
    for (int c = 0; c < ncol; ++c) m->col_start[c + 1] += m->col_start[c];
    m->sites.resize(N);
    m->pos.resize(N);
    {
        std::vector<int> fillc(m->col_start.begin(), m->col_start.end() - 1);
        for (int i = 0; i < N; ++i) m->sites[fillc[colour[i]]++] = i;
        for (int k = 0; k < N; ++k) m->pos[m->sites[k]] = k;
    }
    const std::vector<int> &pos = m->pos, &sites = m->sites;

    // ---------------------------------------------------------------- site classes
    if (dim > 1) {
        // site classes: anisotropy vector and spin length |S|
        int rc = onsite_classes(p, dim, N, sites, &m->stype, &m->dtab, &m->ndc, &m->has_d, err);
        if (rc != MCS_OK) return rc;
    } else {
        ClassTable<1 + MCS_MAXC> tcls;
        std::vector<std::vector<int>> tcount;
        std::vector<double> tS;
        m->stype.assign(N, 0);
        for (int k = 0; k < N; ++k) {
            int i = sites[k];
            double key[1 + MCS_MAXC] = {};
            key[0] = fabs(p->init_spin[i]);
            for (int l = 0; l < p->nlink[i]; ++l) key[1 + linkcls[(size_t)i * z + l]] += 1.0;
            const int t = tcls.find_or_add(key);
            if (t >= MCS_MAXT) FAIL(MCS_EUNSUPPORTED, "Ising model with more than 4 site types");
            if (t == (int)tS.size()) {
                tS.push_back(key[0]);
                std::vector<int> cnt(MCS_MAXC, 0);
                for (int c = 0; c < MCS_MAXC; ++c) cnt[c] = (int)key[1 + c];
                tcount.push_back(cnt);
            }
            m->stype[k] = (uint8_t)t;
        }
        m->ntype = (int)tS.size();
        int base = 0;
        for (int t = 0; t < m->ntype; ++t) {
            m->Stype[t] = tS[t];
            m->ibase[t] = base;
            int stride[MCS_MAXC], ne = 1;
            for (int c = 0; c < MCS_MAXC; ++c) { stride[c] = ne; ne *= (tcount[t][c] + 1); }
            if (ne > 4096) FAIL(MCS_EUNSUPPORTED, "Ising acceptance table too large");
            for (int e = 0; e < ne; ++e) {
                int rem = e, ncv[MCS_MAXC];
                double sumq = 0.0;
                for (int c = 0; c < MCS_MAXC; ++c) {
                    int np = rem % (tcount[t][c] + 1);
                    rem /= (tcount[t][c] + 1);
                    ncv[c] = 2 * np - tcount[t][c];
                    sumq += m->Q[c] * ncv[c];
                }
                IsEntry en;
                memset(&en, 0, sizeof en);
                for (int sg = 0; sg < 2; ++sg) {
                    double sigma = sg ? 1.0 : -1.0;
                    double corr = 2 * (sigma * sumq - p->h * tS[t] * sigma);
                    unsigned long long thr;
                    if (corr >= 0) thr = 1ULL << 32;
                    else {
                        double x = ceil(exp(corr) * 4294967296.0);
                        thr = x >= 4294967296.0 ? (1ULL << 32) : (unsigned long long)x;
                    }
                    en.thr[sg] = thr;
                }
                en.nc = (ncv[0] & 0xff) | ((ncv[1] & 0xff) << 8) | ((ncv[2] & 0xff) << 16) | ((ncv[3] & 0xff) << 24);
                m->itab.push_back(en);
            }
            // per-link code = stride of its class
            (void)stride;
            base += ne;
        }
        // link codes per (site, link)
        // Wolff add thresholds: corr = Q sigma_i sigma_j; add iff corr<0 and 1-exp(2corr) > U
        for (int c = 0; c < m->nclass; ++c)
            for (int sg = 0; sg < 2; ++sg) {
                double corr = sg ? m->Q[c] : -m->Q[c];
                unsigned long long thr = 0;
                if (corr < 0) {
                    double x = ceil((1 - exp(2 * corr)) * 4294967296.0);
                    thr = x >= 4294967296.0 ? (1ULL << 32) : (unsigned long long)x;
                }
                m->wthr[c][sg] = thr;
            }
        // exactness of the incremental bookkeeping: no self links, and every
        // directed link i->j of class c has a reverse link j->i of class c
        bool ok = true;
        for (int i = 0; i < N && ok; ++i)
            for (int l = 0; l < p->nlink[i] && ok; ++l) {
                const int j = p->linked_orb[(size_t)i * z + l];
                const int c = linkcls[(size_t)i * z + l];
                if (j == i) { ok = false; break; }
                bool rev = false;
                for (int q = 0; q < p->nlink[j] && !rev; ++q)
                    rev = p->linked_orb[(size_t)j * z + q] == i && linkcls[(size_t)j * z + q] == c;
                ok = rev;
            }
        m->exact_ok = ok ? 1 : 0;
        }
    // the Ising square rule needs one site type (one acceptance table)
    if (dim == 1 && m->geom == MCS_GEOM_SQUARE && m->ntype != 1) m->geom = MCS_GEOM_ELL;

    // per-link codes in sweep-index space
    if (dim == 1) {
        // stride of a class for each type
        std::vector<std::vector<int>> tstride(m->ntype, std::vector<int>(MCS_MAXC, 0));
        {
            // recompute counts per type from the table sizes
            std::vector<std::vector<int>> cnt(m->ntype, std::vector<int>(MCS_MAXC, 0));
            std::vector<char> seen(m->ntype, 0);
            for (int k = 0; k < N; ++k) {
                int t = m->stype[k];
                if (seen[t]) continue;
                seen[t] = 1;
                int i = sites[k];
                for (int l = 0; l < p->nlink[i]; ++l) cnt[t][linkcls[(size_t)i * z + l]]++;
            }
            for (int t = 0; t < m->ntype; ++t) {
                int s = 1;
                for (int c = 0; c < MCS_MAXC; ++c) { tstride[t][c] = s; s *= cnt[t][c] + 1; }
            }
        }
        if (m->geom == MCS_GEOM_SQUARE)
            for (int d = 0; d < 4; ++d) m->sq_code[d] = tstride[0][m->sq_cls[d]];
        if (m->geom == MCS_GEOM_ELL || true) {
            m->lcode.assign((size_t)std::max(z, 1) * N, 0);
            m->lcls.assign((size_t)std::max(z, 1) * N, 0);
        }
        for (int k = 0; k < N; ++k) {
            int i = sites[k], t = m->stype[k];
            for (int l = 0; l < p->nlink[i]; ++l) {
                int c = linkcls[(size_t)i * z + l];
                m->lcode[(size_t)l * N + k] = (uint16_t)tstride[t][c];
                m->lcls[(size_t)l * N + k] = (uint8_t)c;
            }
        }
    } else if (m->geom != MCS_GEOM_SQUARE) {
        m->lcode.assign((size_t)std::max(z, 1) * N, 0);
        for (int k = 0; k < N; ++k) {
            int i = sites[k];
            for (int l = 0; l < p->nlink[i]; ++l) m->lcode[(size_t)l * N + k] = (uint16_t)linkcls[(size_t)i * z + l];
        }
    }
    if (m->geom == MCS_GEOM_SQUARE && dim > 1) m->lcode.clear();  // neighbours and classes are arithmetic
    m->nbr.assign(m->geom == MCS_GEOM_SQUARE ? 0 : (size_t)std::max(z, 1) * N, 0);
    m->deg.assign(m->geom == MCS_GEOM_SQUARE ? 0 : N, 0);
    for (int k = 0; k < N && m->geom != MCS_GEOM_SQUARE; ++k) {
        int i = sites[k];
        m->deg[k] = (uint8_t)p->nlink[i];
        for (int l = 0; l < p->nlink[i]; ++l) m->nbr[(size_t)l * N + k] = pos[p->linked_orb[(size_t)i * z + l]];
    }

    // ---------------------------------------------------------------- measurement lists
    m->nlat = p->n_lat;
    m->cpair.resize(2 * (size_t)p->n_lat);
    for (int k = 0; k < 2 * p->n_lat; ++k) m->cpair[k] = pos[p->corr_pair[k]];
    m->n_rorb = p->n_rorb;
    m->ncl = p->n_in_cluster;
    m->rorb.resize(p->n_rorb);
    m->rindex.assign(N, -1);
    m->rcl.resize((size_t)p->n_rorb * p->n_in_cluster);
    m->rlink.assign((size_t)p->n_rorb * std::max(z, 1), -1);
    m->rdeg.resize(p->n_rorb);
    if (dim > 1) m->rjc.assign((size_t)p->n_rorb * std::max(z, 1), 0);
    else m->rK.assign((size_t)p->n_rorb * std::max(z, 1), 0.0);
    for (int v = 0; v < p->n_rorb; ++v) {
        int j = p->r_orb[v];
        m->rorb[v] = pos[j];
        m->rindex[pos[j]] = v;
        for (int k = 0; k < p->n_in_cluster; ++k)
            m->rcl[(size_t)v * p->n_in_cluster + k] = pos[p->r_cluster[(size_t)v * p->n_in_cluster + k]];
        m->rdeg[v] = (uint8_t)p->nlink[j];
        for (int l = 0; l < p->nlink[j]; ++l) {
            int t = p->r_link ? p->r_link[(size_t)v * z + l] : -1;
            m->rlink[(size_t)v * z + l] = t < 0 ? -1 : pos[t];
            if (dim > 1) m->rjc[(size_t)v * z + l] = (uint16_t)linkcls[(size_t)j * z + l];
            else m->rK[(size_t)v * z + l] = p->link_strength[(size_t)j * z + l];
        }
    }
    m->rtgt.assign((size_t)p->n_rorb * std::max(z, 1), -1);
    for (int v = 0; v < p->n_rorb; ++v)
        for (int l = 0; l < std::max(z, 1); ++l) {
            int t = m->rlink[(size_t)v * std::max(z, 1) + l];
            m->rtgt[(size_t)v * std::max(z, 1) + l] = t < 0 ? -1 : m->rindex[t];
        }
    m->sflag.assign(N, 0);
    m->pair_identity = 1;
    for (int v = 0; v < p->n_lat; ++v) {
        int a = m->cpair[2 * v], b = m->cpair[2 * v + 1];
        if (a != b || (m->sflag[a] & 1)) m->pair_identity = 0;
        m->sflag[a] |= 1;
    }
    for (int v = 0; v < p->n_rorb; ++v) m->sflag[m->rorb[v]] |= 2;
    if (!m->pair_identity)
        for (int k = 0; k < N; ++k) m->sflag[k] &= 2;
    if (dim == 1) {
        // integer fast path of the Ising frame: one |S| and <= 4 rK values
        std::map<double, int> kc;
        m->rkc.assign(m->rK.size(), 0);
        bool ok = m->ntype == 1;
        for (int v = 0; v < p->n_rorb && ok; ++v)
            for (int l = 0; l < m->rdeg[v]; ++l) {
                double k = m->rK[(size_t)v * std::max(z, 1) + l];
                auto it = kc.find(k);
                int c;
                if (it == kc.end()) {
                    c = (int)kc.size();
                    if (c >= 4) { ok = false; break; }
                    kc[k] = c;
                    m->rKv[c] = k;
                } else c = it->second;
                m->rkc[(size_t)v * std::max(z, 1) + l] = (uint8_t)c;
            }
        for (int k = 0; k < N && ok; ++k) ok = fabs(p->init_spin[k]) == fabs(p->init_spin[0]);
        m->is_fast = ok ? 1 : 0;
    }
    m->ci = m->cj = m->cij = 0;
    for (int v = 0; v < p->n_lat; ++v) {
        bool a = m->rindex[m->cpair[2 * v]] >= 0, b = m->rindex[m->cpair[2 * v + 1]] >= 0;
        m->ci += a; m->cj += b; m->cij += a && b;
    }
    m->ncirc = dim == 3 ? p->n_circuits : 0;
    m->circ.resize(3 * (size_t)m->ncirc);
    for (int k = 0; k < 3 * m->ncirc; ++k) m->circ[k] = pos[p->circuits[k]];
    m->ngroup = dim > 1 ? p->n_group : 0;
    m->gmask.assign(N, 0);
    for (int g = 0; g < m->ngroup; ++g)
        for (int k = 0; k < p->max_group; ++k) {
            int id = p->group_list[(size_t)g * p->max_group + k];
            if (id < 0) break;
            m->gmask[pos[id]] |= (uint8_t)(1u << g);
        }
    m->gall = 0;
    for (int g = 0; g < m->ngroup; ++g) {
        bool all = true;
        for (int k = 0; k < N && all; ++k) all = (m->gmask[k] >> g) & 1;
        if (all) m->gall |= 1 << g;
    }
    m->slen.resize(N);
    m->sval.resize(N);
    for (int k = 0; k < N; ++k) { m->slen[k] = (float)fabs(p->init_spin[sites[k]]); m->sval[k] = (float)p->init_spin[sites[k]]; }

    // ---------------------------------------------------------------- cluster schedule eligibility
    // square lattice, pairs (v, v), chosen sites = even rows x even columns in
    // site order with the four-site block (x,y),(x,y+1),(x+1,y),(x+1,y+1),
    // circuits listed cell by cell inside rows x and x+1, one site class.
    m->cluster_ok = 0;
    if (m->geom == MCS_GEOM_SQUARE && dim > 1 && m->pair_identity && m->ndc == 1 && m->ncl == 4) {
        const int Lx = m->Lx, Ly = m->Ly;
        bool ok = p->n_rorb == (Lx / 2) * (Ly / 2);
        for (int r = 0; r < p->n_rorb && ok; ++r) {
            int x = 2 * (r / (Ly / 2)), y = 2 * (r % (Ly / 2));
            if (p->r_orb[r] != x * Ly + y) { ok = false; break; }
            int want[4] = {x * Ly + y, x * Ly + (y + 1) % Ly, ((x + 1) % Lx) * Ly + y, ((x + 1) % Lx) * Ly + (y + 1) % Ly};
            for (int k = 0; k < 4; ++k)
                if (p->r_cluster[(size_t)r * 4 + k] != want[k]) { ok = false; break; }
        }
        if (ok && m->ncirc > 0) {
            ok = (m->ncirc % N) == 0;
            const int per = ok ? m->ncirc / N : 0;
            // circuit ci belongs to cell ci / per, in row x = cell / Ly; each of
            // its sites must lie in row x or the next one (ids x*Ly .. x*Ly+Ly-1
            // or the next row's), compared as unsigned offsets from the rows' first ids
            for (int x = 0, ci = 0; x < Lx && ok; ++x) {
                const unsigned lo0 = (unsigned)(x * Ly), lo1 = (unsigned)(((x + 1) % Lx) * Ly);
                const int end = (x + 1) * Ly * per;
                for (; ci < end && ok; ++ci)
                    for (int k = 0; k < 3; ++k) {
                        const unsigned id = (unsigned)p->circuits[3 * ci + k];
                        if (id - lo0 >= (unsigned)Ly && id - lo1 >= (unsigned)Ly) { ok = false; break; }
                    }
            }
            for (int k = 0; k < N && ok; ++k) ok = m->slen[k] == m->slen[0] && m->slen[0] > 0;
        }
        for (int g = 4; g < m->ngroup && ok; ++g) ok = (m->gall >> g) & 1;
        m->cluster_ok = ok ? 1 : 0;
    }
    m->meas_regular = 0;
    if (m->cluster_ok) {
        const int Lx = m->Lx, Ly = m->Ly, hb = Ly / 2;
        bool ok = m->ngroup == 0 || m->gall == (1 << m->ngroup) - 1;
        for (int k = 0; k < N && ok; ++k) ok = (m->sflag[k] & 1) && m->sval[k] == m->sval[0];
        int dc[4] = {-1, -1, -1, -1};
        const int zz = std::max(z, 1);
        for (int r = 0; r < p->n_rorb && ok; ++r) {
            const int x = 2 * (r / hb), y = 2 * (r % hb);
            if (m->rdeg[r] != 4) { ok = false; break; }
            const int want[4] = {(((x + 2) % Lx) / 2) * hb + y / 2, (((x - 2 + Lx) % Lx) / 2) * hb + y / 2,
                                 (x / 2) * hb + ((y + 2) % Ly) / 2, (x / 2) * hb + ((y - 2 + Ly) % Ly) / 2};
            int seen = 0;
            for (int l = 0; l < 4 && ok; ++l) {
                const int t = m->rtgt[(size_t)r * zz + l];
                int d = -1;
                for (int q = 0; q < 4; ++q)
                    if (t == want[q] && !(seen & (1 << q))) { d = q; break; }
                if (d < 0) { ok = false; break; }
                seen |= 1 << d;
                const int cls = m->rjc[(size_t)r * zz + l];
                if (dc[d] < 0) dc[d] = cls;
                else if (dc[d] != cls) ok = false;
            }
        }
        if (ok) {
            m->meas_regular = 1;
            for (int d = 0; d < 4; ++d) m->rdir_cls[d] = dc[d];
        }
    }

    // Ising: the cluster schedule's integer frame needs the same regular
    // renormalisation (2x2 blocks on even rows and columns, every site its own
    // correlated pair) with the fast path's classes, and the list slot of
    // each direction's renormalised link (the tie-break of a link's majority
    // is keyed by its slot) the same at every chosen site of one of four
    // kinds: first row or not, first column or not (the reference's builder
    // lists a boundary site's links in another order)
    if (dim == 1 && m->geom == MCS_GEOM_SQUARE && m->is_fast && m->ntype == 1 && m->pair_identity &&
        p->n_lat == N && m->ncl == 4 && m->ngroup == 0) {
        const int Lx = m->Lx, Ly = m->Ly, hb = Ly / 2, zz = std::max(z, 1);
        bool ok = p->n_rorb == (Lx / 2) * hb;
        for (int k = 0; k < N && ok; ++k) ok = (m->sflag[k] & 1) != 0;
        for (int r = 0; r < p->n_rorb && ok; ++r) {
            const int x = 2 * (r / hb), y = 2 * (r % hb);
            if (p->r_orb[r] != x * Ly + y) { ok = false; break; }
            const int want[4] = {x * Ly + y, x * Ly + (y + 1) % Ly, ((x + 1) % Lx) * Ly + y, ((x + 1) % Lx) * Ly + (y + 1) % Ly};
            for (int k = 0; k < 4; ++k)
                if (p->r_cluster[(size_t)r * 4 + k] != want[k]) { ok = false; break; }
        }
        int slot[16], kc[4] = {-1, -1, -1, -1};
        for (int k = 0; k < 16; ++k) slot[k] = -1;
        for (int r = 0; r < p->n_rorb && ok; ++r) {
            const int x = 2 * (r / hb), y = 2 * (r % hb), kind = (x == 0 ? 1 : 0) | (y == 0 ? 2 : 0);
            if (m->rdeg[r] != 4) { ok = false; break; }
            const int want[4] = {(((x + 2) % Lx) / 2) * hb + y / 2, (((x - 2 + Lx) % Lx) / 2) * hb + y / 2,
                                 (x / 2) * hb + ((y + 2) % Ly) / 2, (x / 2) * hb + ((y - 2 + Ly) % Ly) / 2};
            int seen = 0;
            for (int l = 0; l < 4 && ok; ++l) {
                const int t = m->rtgt[(size_t)r * zz + l];
                int d = -1;
                for (int q = 0; q < 4; ++q)
                    if (t == want[q] && !(seen & (1 << q))) { d = q; break; }
                if (d < 0) { ok = false; break; }
                seen |= 1 << d;
                const int cls = m->rkc[(size_t)r * zz + l];
                if (slot[4 * kind + d] < 0) slot[4 * kind + d] = l;
                else if (slot[4 * kind + d] != l) ok = false;
                if (kc[d] < 0) kc[d] = cls;
                else if (kc[d] != cls) ok = false;
            }
        }
        for (int k = 0; k < 16 && ok; ++k) ok = slot[k] >= 0;  // every kind of chosen site occurs
        if (ok) {
            m->cluster_ok = 1;
            for (int k = 0; k < 16; ++k) m->rdir_slot[k] = slot[k];
            for (int d = 0; d < 4; ++d) m->rdir_cls[d] = kc[d];
        }
    }

    if (dim > 1) m->linkcls = std::move(linkcls);
    return compile_program_state(p, o, m, dim, err);
}

// The sweep program (units, measurement interval, frames) and the initial
// state of a compiled model (sweep order m->sites / m->pos).
static int compile_program_state(const mcs_problem *p, const mcs_options *o, HostModel *m, int dim, std::string *err)
{
    const int N = p->n_sites;
    const std::vector<int> &pos = m->pos, &sites = m->sites;
    // ---------------------------------------------------------------- program
    if (p->algorithm == 0) {
        m->upm = (int)std::min<long long>((p->ninterval + N - 1) / N, 1 << 30);
    } else {
        if (p->ninterval > (1 << 30)) FAIL(MCS_EINVAL, "ninterval too large for Wolff");
        m->upm = (int)p->ninterval;
    }
    m->nsweep = p->nsweep;
    m->units_thermal = p->nthermal * (long long)m->upm;
    m->units_total = m->units_thermal + p->nsweep * (long long)m->upm;
    m->frames = p->spin_frames;
    m->frame_every = p->spin_frames > 0 ? p->nsweep / p->spin_frames : 1;
    if (m->frame_every < 1) m->frame_every = 1;
    const bool rnd = o && o->random_init;
    m->offset_energy = (o && o->absolute_energy) ? 0 : 1;

    // ---------------------------------------------------------------- initial state
    m->device_random_init = rnd ? 1 : 0;  // drawn on the device by the initial-state kernel
    if (dim == 1) {
        m->init_sigma.resize(N);
        double M0 = 0, first = 0;
        for (int k = 0; k < N; ++k) {
            int i = sites[k];
            int8_t sg = p->init_spin[i] < 0 ? -1 : 1;
            m->init_sigma[k] = sg;
            M0 += fabs(p->init_spin[i]) * sg;
        }
        long long nfirst = std::min<long long>(p->ninterval, N);
        for (long long i = 0; i < nfirst; ++i) first += p->init_spin[i];
        int lastk = pos[N - 1];
        double slast0 = fabs(p->init_spin[N - 1]) * m->init_sigma[lastk];
        m->last_site = lastk;
        if (rnd) {
            m->ts_const = 0.0;
            m->ts_wolff_last = 0;
        } else if (p->algorithm == 0) {
            m->ts_const = M0 - first;
            m->ts_wolff_last = 0;
        } else {
            m->ts_const = M0 - slast0 - first;
            m->ts_wolff_last = 1;
        }
    } else {
        m->init_vec.assign((size_t)3 * N, 0.f);
        for (int k = 0; k < N; ++k) {
            int i = sites[k];
            double S0 = p->init_spin[i];
            double v[3] = {S0, 0, 0}, d[3];
            uint32_t w[4];
            if (rnd || p->flunc == 0.0) {
                // (S,0,0) normalised and scaled back is (S,0,0); random states are drawn on the device
                m->init_vec[k] = (float)S0;
                continue;
            } else {
                philox_host((uint32_t)k, 0, 0, 0x4000u, m->seed, w);
                eng_dir(dim, w[0], w[1], d);
                v[0] += d[0] * p->flunc; v[1] += d[1] * p->flunc;
                if (dim == 3) v[2] += d[2] * p->flunc;
            }
            double len = dim == 3 ? sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) : sqrt(v[0] * v[0] + v[1] * v[1]);
            if (len >= 1e-5) { v[0] /= len; v[1] /= len; if (dim == 3) v[2] /= len; }
            double a = fabs(S0);
            for (int c = 0; c < 3; ++c) {
                double x = (c < dim) ? v[c] * a : 0.0;
                m->init_vec[(size_t)c * N + k] = (float)x;
            }
        }
        m->last_site = pos[N - 1];
    }
    return MCS_OK;
}

}  // namespace mcs
