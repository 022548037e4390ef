// lg_problem.h -- host-side Sedov problem description (the Domain's inputs).
//
// Built once on the host, exactly as Domain::Domain does for one rank
// (lulesh-init.cc:16-194), then uploaded.  The arrays keep the reference's
// names and layouts so that the Domain accessor surface maps 1:1 onto them.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "lg_device.h"

namespace lg {


// Physics constants, lulesh-init.cc:20-38.  hgcoef is the only one the
// variants change.
struct Constants {
    double e_cut = 1.0e-7, p_cut = 1.0e-7, q_cut = 1.0e-7, v_cut = 1.0e-10, u_cut = 1.0e-7;
    double hgcoef = 3.0, ss4o3 = 4.0 / 3.0, qstop = 1.0e+12, monoq_max_slope = 1.0;
    double monoq_limiter_mult = 2.0, qlc_monoq = 0.5, qqc_monoq = 2.0 / 3.0, qqc = 2.0;
    double eosvmax = 1.0e+9, eosvmin = 1.0e-9, pmin = 0.0, emin = -1.0e+15;
    double dvovmax = 0.1, refdens = 1.0;
};

// Time-step state, lulesh-init.cc:146-156 and 192.
struct TimeState {
    double time = 0.0, deltatime = 0.0, dtcourant = 1.0e+20, dthydro = 1.0e+20;
    double stoptime = 1.0e-2, dtmax = 1.0e-2, dtfixed = -1.0e-6;
    double deltatimemultlb = 1.1, deltatimemultub = 1.2;
    int cycle = 0;
};

struct Problem {
    int nx = 0, numElem = 0, numNode = 0, numReg = 0, balance = 1, cost = 1;
    Constants k;
    TimeState t;
    // node-centred
    std::vector<double> x, y, z, xd, yd, zd, xdd, ydd, zdd, fx, fy, fz, nodalMass;
    std::vector<int> symmX, symmY, symmZ;
    // element-centred
    std::vector<int> nodelist, lxim, lxip, letam, letap, lzetam, lzetap, elemBC;
    std::vector<double> e, p, q, ql, qq, v, volo, vnew, delv, vdov, arealg, ss, elemMass;
    std::vector<int> regNumList, regElemSize;
    std::vector<std::vector<int>> regElemlist;
    // node -> element-corner CSR, lulesh-init.cc:272-337
    std::vector<int> nodeElemStart, nodeElemCornerList;
};

// The glibc random() TYPE_3 additive-feedback generator behind the
// reference's srand(0)/rand() region draw (lulesh-init.cc:408-480),
// restated from its published description so that set-up neither touches
// nor depends on the process-wide libc generator.
class GlibcRand {
  public:
    explicit GlibcRand(unsigned seed);
    int next();

  private:
    int32_t r_[34];
    int i_ = 0;
};

// Domain::Domain for one rank (col=row=plane=0, tp=1).  hgcoef replaces the
// constant of lulesh-init.cc:25; einit_factor scales the deposited energy of
// lulesh-init.cc:183-189 (and therefore the initial time step of line 192).
Problem build_sedov(int nx, int numReg, int balance, int cost, double hgcoef,
                    double einit_factor);

// The part of build_sedov that stays on the host when the mesh is built on
// the device (lg_setup.cu): sizes, constants, the time-step state (the first
// step from the analytic volume of element 0) and the region draw, which
// follows the reference's sequential random stream.  The mesh and field
// vectors stay empty.
Problem build_sedov_scalars(int nx, int numReg, int balance, int cost, double hgcoef,
                            double einit_factor);

// Deposited origin energy, lulesh-init.cc:183-189.
double sedov_einit(int nx, double einit_factor);

// SetupThreadSupportStructures (lulesh-init.cc:272-337) from p.nodelist.
void build_corner_list(Problem &p);

// Region index sets from p.regNumList (lulesh-init.cc:492-509).
void build_region_sets(Problem &p);

// CalcElemVolume, lulesh.cc:1273-1366 (host copy used by set-up).
double elem_volume_host(const double x[8], const double y[8], const double z[8]);

// EOS repetitions of region r, lulesh.cc:2390-2400.
int region_rep(int r, int numReg, int cost);

// The order in which the material kernels visit the regions: most EOS
// repetitions first, ascending region index among equals.  Every element's
// material update is independent and the dt reduction is a minimum, so the
// order cannot change a result; putting the expensive blocks at the front of
// the grid keeps them from forming a tail that leaves SMs idle.
std::vector<int> region_visit_order(int numReg, int cost);

// The material phase's work items.  Large meshes: one item per element
// (item_rep = the element's EOS repetitions), in region visit order; returns
// false.  When a repeated count's elements number fewer than T = 3/8 of
// `resident` (the threads of one resident wave), the phase runs split
// (k_material_inputs / k_material_eos / k_material_finish) and the items are
// repetition items: each element's repetitions in near-equal shares of at
// most R = max(1, ceil(total repetitions / (4 resident))), its first item
// the writer (item_rep > 0; the others < 0), sorted by share, largest
// first; returns true.
bool build_material_items(const Problem &p, long long resident, std::vector<int> &item_elem,
                          std::vector<int> &item_rep);

// End-of-run report text, lulesh-util.cc:175-230.
std::string format_report(int nx, int cycle, double e0, double maxAbsDiff,
                          double totalAbsDiff, double maxRelDiff, double elapsed);

}  // namespace lg
