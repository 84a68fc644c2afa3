// Host-side construction of a run's initial state and constant geometry.
#ifndef MAHYCO_GB300_INIT_H
#define MAHYCO_GB300_INIT_H

#include <vector>

#include "hydro_gb300.h"

namespace hydro {

// Initial state and Euler geometry of one run, SoA, as host vectors.
// Per-material arrays are nbmat_max(3) planes of nc values.
struct HostInit {
  long long nx = 0, ny = 0, nc = 0, nn = 0;
  // boundary conditions (Cdl, includes/ConditionsLimites.h)
  int bc_left = 0, bc_right = 0, bc_bottom = 0, bc_top = 0;
  double v_left[2] = {0, 1}, v_right[2] = {0, 1}, v_bottom[2] = {1, 0},
         v_top[2] = {1, 0};
  int periodic_x = 0;
  double dt_init = 0.0;
  // geometry
  std::vector<double> xs, ys;        // node coordinates per column / row
  std::vector<double> cqs;           // 8 planes (corner k, component d)
  std::vector<double> s0, sqs0, cflsq;
  std::vector<double> nout;          // 4 planes: L.x, R.x, B.y, T.y
  std::vector<double> flv, flh;      // Euler face lengths per row / column
  // cell state
  std::vector<double> rho, p, c, e, q, divu, cell_mass;
  std::vector<double> rhom, pm, cm, em, qm, fm, mfm, cmassm;  // 3 planes
  std::vector<double> rho0_left;     // initial density of column 0 (periodic)
  std::vector<int> mixte, pure;
  // node state
  std::vector<double> u;             // 2 planes
  std::vector<double> node_mass;
  // Eucclhyd: cell velocity, constant cell and corner geometry of the Euler
  // mesh, per (cell, corner k = position of the node in the cell)
  std::vector<double> uc;            // 2 planes
  std::vector<double> xc;            // 2 planes: cell centroids
  std::vector<double> perim, evol;   // cell perimeter, Euler volume
  std::vector<double> lpc;           // 8 planes [2k + d]: l_pc n_pc
  std::vector<double> cmat;          // 12 planes [3k + e]: corner matrix
                                     // entries 00, 01 (= 10), 11
};

// Builds the initial state for spec (VNR test cases of vnr_remap/Init.cc and
// the extensions selected by spec->init_variant).  Returns 0 or a negative
// status with hydro_last_error() set.
int build_initial_state(const hydro_spec& spec, HostInit& out);

// Eucclhyd set-up (eucclhyd_remap/Init.cc, PhaseLagrange.cc:27-66) for the
// Sod, bi-material Sod, triple-point and Sedov cases.
int build_initial_state_euc(const hydro_spec& spec, HostInit& out);

}  // namespace hydro
#endif
