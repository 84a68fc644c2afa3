// Host part of a run's set-up: option checks, boundary conditions and the
// initial time step where it is a constant.  The initial state and the
// constant Euler geometry are built on the device (kernels/init.cu).
#ifndef MAHYCO_GB300_INIT_H
#define MAHYCO_GB300_INIT_H

#include "hydro_gb300.h"

namespace hydro {

struct HostInit {
  long long nx = 0, ny = 0, nc = 0, nn = 0;
  // boundary conditions (Cdl, includes/ConditionsLimites.h)
  int bc_left = 0, bc_right = 0, bc_bottom = 0, bc_top = 0;
  double v_left[2] = {0, 1}, v_right[2] = {0, 1}, v_bottom[2] = {1, 0},
         v_top[2] = {1, 0};
  int periodic_x = 0;
  // sides whose remap takes a boundary flux (Cdl::left/right/bottom/top
  // FluxBC, remap/BoundaryFluxes.cc): kFlux* bits
  int flux_bc = 0;
  // initial dt_n when it does not come from the initial state (Eucclhyd,
  // VNR without the Lagrange phase); VNR with it reduces over the cells on
  // the device
  double dt_init = 0.0;
  bool dt_from_cells = false;
};

// VNR test cases of vnr_remap/Init.cc and the extensions selected by
// spec->init_variant.  Returns 0 or a negative status with
// hydro_last_error() set.
int init_options(const hydro_spec& spec, HostInit& out);

// Eucclhyd set-up (eucclhyd_remap/Init.cc) for the Sod, bi-material Sod,
// triple-point, Sedov, Noh, shock-bubble and unit test cases.
int init_options_euc(const hydro_spec& spec, HostInit& out);

}  // namespace hydro
#endif
