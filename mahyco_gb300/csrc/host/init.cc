// Host part of a VNR run's set-up (vnr_remap/Init.cc:10-64
// initBoundaryConditions; the checks of Vnr::init's test-case switch).  The
// state and geometry of Vnr::simulate's set-up sequence (VnrRemap.cc
// :330-341) are built on the device by kernels/init.cu.
#include "init.h"

#include <string>

#include "../internal.h"

namespace hydro {
namespace {

int init_bc(const hydro_spec& s, HostInit& h) {
  const int t = s.test_case;
  if (t == 4 || t == 15 || t == 5 || t == 16) {
    // Sod / BiSod (vnr_remap/Init.cc:10-37): walls
    h.bc_left = h.bc_right = h.bc_top = h.bc_bottom = kBcSym;
  } else if (t == 1) {
    // Sedov (extension for VNR): the boundary conditions of the Eucclhyd
    // Sedov case (eucclhyd_remap/Init.cc:47-64): symmetry on the left and
    // bottom, zero imposed velocity on the right and top
    h.bc_left = kBcSym;
    h.bc_bottom = kBcSym;
    h.bc_right = kBcImposed;
    h.v_right[0] = 0.0;
    h.v_right[1] = 0.0;
    h.bc_top = kBcImposed;
    h.v_top[0] = 0.0;
    h.v_top[1] = 0.0;
  } else if (t == 7 || t == 18 || t == 9 || t == 20) {
    // Advection X (Init.cc:38-50)
    h.bc_right = kBcImposed;
    h.v_right[0] = 1.0;
    h.v_right[1] = 0.0;
    h.periodic_x = 1;
    h.bc_left = kBcImposed;
    h.v_left[0] = 1.0;
    h.v_left[1] = 0.0;
    h.bc_top = kBcSym;
    h.bc_bottom = kBcSym;
  } else if (t == 0 || t == 11) {
    // UnitTestCase / BiUnitTestCase (Init.cc:65-93): velocity (1, 0)
    // imposed on every side, a flux condition on the left
    h.bc_right = kBcImposed;
    h.v_right[0] = 1.0;
    h.v_right[1] = 0.0;
    h.bc_left = kBcImposed;
    h.v_left[0] = 1.0;
    h.v_left[1] = 0.0;
    h.flux_bc = kFluxLeft;
    h.bc_bottom = kBcImposed;
    h.v_bottom[0] = 1.0;
    h.v_bottom[1] = 0.0;
    h.bc_top = kBcImposed;
    h.v_top[0] = 1.0;
    h.v_top[1] = 0.0;
  } else if (t == 8 || t == 19) {
    // Advection Y (Init.cc:51-64)
    h.bc_bottom = kBcImposed;
    h.v_bottom[0] = 0.0;
    h.v_bottom[1] = 1.0;
    h.bc_top = kBcImposed;
    h.v_top[0] = 0.0;
    h.v_top[1] = 1.0;
    h.bc_left = kBcSym;
    h.bc_right = kBcSym;
  } else {
    return fail(-10, "VNR initialisation: test case " + std::to_string(t) +
                         " is not a VNR test case");
  }
  return 0;
}

}  // namespace

int init_options(const hydro_spec& s, HostInit& h) {
  if (s.scheme != HYDRO_SCHEME_VNR) return fail(-11, "not a VNR run");
  if (s.nx < 2 || s.ny < 2) return fail(-12, "nx and ny must be >= 2");
  const int t = s.test_case;
  const bool advection = (t == 7 || t == 8 || t == 18 || t == 19 || t == 20 || t == 21);
  if (!(t == 4 || t == 5 || t == 15 || t == 16 || t == 1 || t == 0 || t == 11 || advection))
    return fail(-10, "VNR initialisation: unsupported test case");
  h.nx = s.nx;
  h.ny = s.ny;
  h.nc = (long long)s.nx * s.ny;
  h.nn = (long long)(s.nx + 1) * (s.ny + 1);
  if (int rc = init_bc(s, h)) return rc;
  // initDeltaT (Init.cc:435-457) runs with the Lagrange phase only
  h.dt_from_cells = (s.sans_lagrange == 0);
  h.dt_init = h.dt_from_cells ? 0.0 : s.dt_init;
  return 0;
}

}  // namespace hydro
