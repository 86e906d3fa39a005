// mcs_model.h -- host-side model compiler: from the reference's flattened
// MCMainFunction arrays to the engine's device layout.
#pragma once
#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/mcsgpu.h"
#include "mcs_internal.h"

namespace mcs {

struct HostModel {
    // identity
    int model = 0, dim = 0, alg = 0, N = 0, zmax = 0;
    int geom = MCS_GEOM_ELL;
    int Lx = 0, Ly = 0;
    int ncol = 0;
    std::vector<int> col_start;          // ncol+1
    std::vector<int> sites;              // sweep index -> original site
    std::vector<int> pos;                // original site -> sweep index
    // ELL (sweep-index space, [zmax][N])
    std::vector<int> nbr;
    std::vector<uint16_t> lcode;
    std::vector<uint8_t> lcls;
    std::vector<uint8_t> deg;
    int sq_code[4] = {0, 0, 0, 0};
    int sq_cls[4] = {0, 0, 0, 0};
    std::vector<uint8_t> stype;          // per sweep index
    // O(n) tables
    std::vector<float> jtab;             // [njc][9]
    std::vector<double> jtab64;
    int njc = 0, fullJ = 0;
    std::vector<float> dtab;             // [ndc][4]: Dx, Dy, Dz, |S|
    int ndc = 0, has_d = 0;
    // Ising tables
    std::vector<IsEntry> itab;
    int ntype = 0, nclass = 0, exact_ok = 0;
    int ibase[MCS_MAXT] = {0, 0, 0, 0};
    double Q[MCS_MAXC] = {0, 0, 0, 0};
    double Stype[MCS_MAXT] = {0, 0, 0, 0};
    unsigned long long wthr[MCS_MAXC][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
    double h = 0.0, flunc = 0.0;
    // measurement lists (sweep indices)
    std::vector<int> cpair, rorb, rcl, rlink, rindex, circ;
    std::vector<uint16_t> rjc;
    std::vector<double> rK;
    std::vector<uint8_t> rkc;
    double rKv[4] = {0, 0, 0, 0};
    int is_fast = 0;
    std::vector<uint8_t> rdeg, gmask;
    std::vector<float> slen, sval;
    std::vector<uint8_t> sflag;
    std::vector<int> rtgt;
    int pair_identity = 0;
    int gall = 0;
    int cluster_ok = 0;     // the row-split cluster schedule can run this replica
    int meas_regular = 0;   // cluster frame from arithmetic (see Rep::meas_regular)
    int rdir_cls[4] = {0, 0, 0, 0};
    int rdir_slot[16] = {};  // Ising: list slot of the renormalised link of each direction, by kind of chosen site
    int nlat = 0, n_rorb = 0, ncl = 0, ncirc = 0, ngroup = 0;
    int ci = 0, cj = 0, cij = 0;
    // program
    long long units_thermal = 0, units_total = 0, nsweep = 0;
    int upm = 1;
    int frames = 0;
    long long frame_every = 1;
    double ts_const = 0.0;
    int ts_wolff_last = 0, last_site = 0, offset_energy = 1;
    // initial state (sweep order)
    std::vector<int8_t> init_sigma;      // Ising
    std::vector<float> init_vec;         // O(n) [dim][N]
    int device_random_init = 0;          // draw the initial state on the device
    unsigned long long seed = 0;
    // coupling class of every link [N][zmax] (original site order), kept so
    // that a later replica of the same lattice can be checked against it
    std::vector<int> linkcls;
};

// The structural inputs of one O(n) problem (everything but the coupling and
// anisotropy values, the field, the sweep counts and the options), copied, so
// that a later problem can be recognised as the same lattice.
struct StructInputs {
    int model = 0, alg = 0, N = 0, z = 0;
    int n_circuits = 0, n_lat = 0, n_group = 0, max_group = 0, n_rorb = 0, n_in_cluster = 0, ignore_offdiag = 0;
    bool has_rlink = false;
    std::vector<int32_t> nlink, linked_orb, circuits, corr_pair, group_list, r_orb, r_cluster, r_link;
    std::vector<double> init_spin;
};
// A compiled model together with its structural inputs: the template from
// which problems of the same lattice are compiled without redoing the
// geometry, colouring and measurement lists.  The model is stored without
// what every problem recomputes (initial state) and without its link classes,
// which are kept beside it: a problem compiled from the template copies only
// the structure.
struct ModelTemplate {
    HostModel hm;
    StructInputs in;
    std::vector<int> linkcls;   // coupling class of every link, as HostModel::linkcls
};
std::shared_ptr<const ModelTemplate> make_template(const mcs_problem *p, const HostModel &m);

// Returns MCS_OK or an error code with a message in *err.  With a template of
// the same lattice (bitwise equal structural inputs, the same partition of the
// links into coupling classes and of the sites into anisotropy classes) the
// structure is taken from the template and only the values, the program and
// the initial state are compiled; *reused tells which path ran.
int compile_model(const mcs_problem *p, const mcs_options *o, HostModel *m, std::string *err,
                  const ModelTemplate *tmpl = nullptr, bool *reused = nullptr);

// Philox4x32-10 on the host (the device's generator, for initial states).
void philox_host(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, unsigned long long seed, uint32_t out[4]);

}  // namespace mcs
