// mcs_model.h -- host-side model compiler: from the reference's flattened
// MCMainFunction arrays to the engine's device layout.
#pragma once
#include <stdint.h>

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
};

// Returns MCS_OK or an error code with a message in *err.
int compile_model(const mcs_problem *p, const mcs_options *o, HostModel *m, std::string *err);

// Philox4x32-10 on the host (the device's generator, for initial states).
void philox_host(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, unsigned long long seed, uint32_t out[4]);

}  // namespace mcs
