// Host part of a Eucclhyd run's set-up: initBoundaryConditions
// (eucclhyd_remap/Init.cc:15-98) and setUpTimeLoopN's initial time step
// (Init.cc:721-760) for the Sod, bi-material Sod, triple-point, Sedov, Noh,
// shock-bubble and unit test cases.  The state and the corner / cell geometry of
// Eucclhyd::simulate's set-up (EucclhydRemap.cc:273-287) are built on the
// device by kernels/init.cu.
#include <string>

#include "../internal.h"
#include "init.h"

namespace hydro {

int init_options_euc(const hydro_spec& s, HostInit& h) {
  if (s.nx < 2 || s.ny < 2) return fail(-12, "nx and ny must be >= 2");
  h.nx = s.nx;
  h.ny = s.ny;
  h.nc = (long long)s.nx * s.ny;
  h.nn = (long long)(s.nx + 1) * (s.ny + 1);
  const int t = s.test_case;
  // ---- initBoundaryConditions (Init.cc:15-98)
  if (t == 4 || t == 5 || t == 15 || t == 16 || t == 2 || t == 13) {
    h.bc_left = h.bc_right = h.bc_top = h.bc_bottom = kBcSym;
  } else if (t == 1 || t == 12 || t == 6 || t == 17) {
    // Sedov, Noh (Init.cc:47-64, 79-97): symmetry left and bottom, zero
    // imposed velocity right and top
    h.bc_left = kBcSym;
    h.bc_bottom = kBcSym;
    h.bc_right = kBcImposed;
    h.bc_top = kBcImposed;
    h.v_right[0] = h.v_right[1] = 0.0;
    h.v_top[0] = h.v_top[1] = 0.0;
  } else if (t == 14) {
    // BiShockBubble (Init.cc:30-46): the gas comes in from the right at the
    // imposed velocity, and the remap takes the right boundary's flux
    h.bc_left = kBcSym;
    h.bc_right = kBcImposed;
    h.v_right[0] = -124.824;
    h.v_right[1] = 0.0;
    h.bc_top = kBcSym;
    h.bc_bottom = kBcSym;
    h.flux_bc = kFluxRight;
  } else if (t == 0 || t == 11) {
    // UnitTestCase / BiUnitTestCase: no branch of initBoundaryConditions, so
    // every side keeps the Cdl defaults (condition 0, no constraint value)
  } else {
    return fail(-10, "Eucclhyd initialisation: test case " + std::to_string(t) +
                         " is not supported");
  }
  // symmetry values: ey on the left / right sides, ex on top / bottom
  if (h.bc_left == kBcSym) { h.v_left[0] = 0.0; h.v_left[1] = 1.0; }
  if (h.bc_right == kBcSym) { h.v_right[0] = 0.0; h.v_right[1] = 1.0; }
  if (h.bc_top == kBcSym) { h.v_top[0] = 1.0; h.v_top[1] = 0.0; }
  if (h.bc_bottom == kBcSym) { h.v_bottom[0] = 1.0; h.v_bottom[1] = 0.0; }

  // setUpTimeLoopN (Init.cc:729-755): the unit tests have no branch and
  // keep the value-initialised deltat_n, 0 (their first cycle then stops on
  // dt < dt_min, as the reference does)
  h.dt_from_cells = false;
  if (t == 2 || t == 13)
    h.dt_init = 1.0e-5;
  else if (t == 14)
    h.dt_init = 1.0e-7;
  else if (t == 0 || t == 11)
    h.dt_init = 0.0;
  else
    h.dt_init = 1.0e-4;
  return 0;
}

}  // namespace hydro
