// Host part of a Eucclhyd run's set-up: initBoundaryConditions
// (eucclhyd_remap/Init.cc:15-98) and setUpTimeLoopN's initial time step
// (Init.cc:721-760).  The state and the corner / cell geometry of
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
  } else if (t == 1 || t == 12) {
    h.bc_left = kBcSym;
    h.bc_bottom = kBcSym;
    h.bc_right = kBcImposed;
    h.bc_top = kBcImposed;
    h.v_right[0] = h.v_right[1] = 0.0;
    h.v_top[0] = h.v_top[1] = 0.0;
  } else {
    return fail(-10, "Eucclhyd initialisation: test case " + std::to_string(t) +
                         " is not supported");
  }
  // symmetry values: ey on the left / right sides, ex on top / bottom
  if (h.bc_left == kBcSym) { h.v_left[0] = 0.0; h.v_left[1] = 1.0; }
  if (h.bc_right == kBcSym) { h.v_right[0] = 0.0; h.v_right[1] = 1.0; }
  if (h.bc_top == kBcSym) { h.v_top[0] = 1.0; h.v_top[1] = 0.0; }
  if (h.bc_bottom == kBcSym) { h.v_bottom[0] = 1.0; h.v_bottom[1] = 0.0; }

  h.dt_from_cells = false;
  h.dt_init = (t == 2 || t == 13) ? 1.0e-5 : 1.0e-4;
  return 0;
}

}  // namespace hydro
